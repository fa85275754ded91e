//! `ConvTensorExt::conv_tensor_cores`: the direct convolution of `conv` on
//! the GB300 tensor cores (3xBF16 split products accumulated in f32), run by
//! `ndconv_conv_bf16x3`.  No counterpart in the original crate; the results
//! meet the same normwise bound against f64 as `conv` (1e-5), not its
//! rounding.  f32 and `Complex<f32>` only.
use ndarray::{Array, ArrayBase, Data, Dim, Ix, RawData};
use num::Complex;

use crate::device::{convolve, DeviceElem};
use crate::{ConvMode, Error, IntoKernelWithDilation, PaddingMode};

/// Element types the tensor-core path takes.
pub trait TensorElem: DeviceElem {}
impl TensorElem for f32 {}
impl TensorElem for Complex<f32> {}

pub trait ConvTensorExt<'a, T, S, SK, const N: usize>
where
    T: TensorElem,
    S: RawData,
    SK: RawData,
{
    /// Same arguments and output shape as `ConvExt::conv`.
    fn conv_tensor_cores(
        &self,
        kernel: impl IntoKernelWithDilation<'a, SK, N>,
        conv_mode: ConvMode<N>,
        padding_mode: PaddingMode<N, T>,
    ) -> Result<Array<T, Dim<[Ix; N]>>, Error<N>>;
}

impl<'a, T, S, SK, const N: usize> ConvTensorExt<'a, T, S, SK, N> for ArrayBase<S, Dim<[Ix; N]>>
where
    T: TensorElem,
    S: Data<Elem = T> + 'a,
    SK: Data<Elem = T> + 'a,
    Dim<[Ix; N]>: ndarray::Dimension,
    [Ix; N]: ndarray::IntoDimension<Dim = Dim<[Ix; N]>>,
{
    fn conv_tensor_cores(
        &self,
        kernel: impl IntoKernelWithDilation<'a, SK, N>,
        conv_mode: ConvMode<N>,
        padding_mode: PaddingMode<N, T>,
    ) -> Result<Array<T, Dim<[Ix; N]>>, Error<N>> {
        let kernel = kernel.into_kernel_with_dilation();
        convolve(false, self, kernel, conv_mode, padding_mode, |p, x, k, y| unsafe {
            ndarray_conv_sys::ndconv_conv_bf16x3(p, x, k, y, std::ptr::null_mut())
        })
    }
}
