//! `ConvExt::conv`: direct convolution (the original's src/conv/mod.rs
//! trait), run by `ndconv_conv`.
use ndarray::{Array, ArrayBase, Data, Dim, Ix, RawData};

use crate::device::{convolve, DeviceElem};
use crate::{ConvMode, Error, IntoKernelWithDilation, PaddingMode};

pub trait ConvExt<'a, T, S, SK, const N: usize>
where
    T: num::traits::NumAssign + Copy,
    S: RawData,
    SK: RawData,
{
    /// Convolve with `kernel` (an array reference, or one with dilation /
    /// `no_reverse`), output size by `conv_mode`, borders by `padding_mode`.
    fn conv(
        &self,
        kernel: impl IntoKernelWithDilation<'a, SK, N>,
        conv_mode: ConvMode<N>,
        padding_mode: PaddingMode<N, T>,
    ) -> Result<Array<T, Dim<[Ix; N]>>, Error<N>>;
}

impl<'a, T, S, SK, const N: usize> ConvExt<'a, T, S, SK, N> for ArrayBase<S, Dim<[Ix; N]>>
where
    T: DeviceElem,
    S: Data<Elem = T> + 'a,
    SK: Data<Elem = T> + 'a,
    Dim<[Ix; N]>: ndarray::Dimension,
    [Ix; N]: ndarray::IntoDimension<Dim = Dim<[Ix; N]>>,
{
    fn conv(
        &self,
        kernel: impl IntoKernelWithDilation<'a, SK, N>,
        conv_mode: ConvMode<N>,
        padding_mode: PaddingMode<N, T>,
    ) -> Result<Array<T, Dim<[Ix; N]>>, Error<N>> {
        let kernel = kernel.into_kernel_with_dilation();
        convolve(false, self, kernel, conv_mode, padding_mode, |p, x, k, y| unsafe {
            ndarray_conv_sys::ndconv_conv(p, x, k, y, std::ptr::null_mut())
        })
    }
}
