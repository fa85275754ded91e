//! Kernels with dilation and the reverse flag (the original's
//! `with_dilation`, `reverse` / `no_reverse`): only recorded here, the
//! library applies them as the tap stride and the kernel read order.
use ndarray::{ArrayBase, Dim, Ix, RawData};

/// A kernel view with its per-axis dilation and whether it is flipped
/// (convolution, the default) or not (correlation).
pub struct KernelWithDilation<'a, S: RawData, const N: usize> {
    pub(crate) kernel: &'a ArrayBase<S, Dim<[Ix; N]>>,
    pub(crate) dilation: [usize; N],
    pub(crate) reverse: bool,
}

/// A dilation for every axis (`usize`) or per axis (`[usize; N]`).
pub trait IntoDilation<const N: usize> {
    fn into_dilation(self) -> [usize; N];
}

impl<const N: usize> IntoDilation<N> for usize {
    fn into_dilation(self) -> [usize; N] {
        [self; N]
    }
}

impl<const N: usize> IntoDilation<N> for [usize; N] {
    fn into_dilation(self) -> [usize; N] {
        self
    }
}

pub trait WithDilation<S: RawData, const N: usize> {
    fn with_dilation(&self, dilation: impl IntoDilation<N>) -> KernelWithDilation<'_, S, N>;
}

impl<S: RawData, const N: usize> WithDilation<S, N> for ArrayBase<S, Dim<[Ix; N]>> {
    fn with_dilation(&self, dilation: impl IntoDilation<N>) -> KernelWithDilation<'_, S, N> {
        KernelWithDilation { kernel: self, dilation: dilation.into_dilation(), reverse: true }
    }
}

pub trait IntoKernelWithDilation<'a, S: RawData, const N: usize> {
    fn into_kernel_with_dilation(self) -> KernelWithDilation<'a, S, N>;
}

impl<'a, S: RawData, const N: usize> IntoKernelWithDilation<'a, S, N> for &'a ArrayBase<S, Dim<[Ix; N]>> {
    fn into_kernel_with_dilation(self) -> KernelWithDilation<'a, S, N> {
        KernelWithDilation { kernel: self, dilation: [1; N], reverse: true }
    }
}

impl<'a, S: RawData, const N: usize> IntoKernelWithDilation<'a, S, N> for KernelWithDilation<'a, S, N> {
    fn into_kernel_with_dilation(self) -> KernelWithDilation<'a, S, N> {
        self
    }
}

pub trait ReverseKernel<'a, S: RawData, const N: usize> {
    fn reverse(self) -> KernelWithDilation<'a, S, N>;
    fn no_reverse(self) -> KernelWithDilation<'a, S, N>;
}

impl<'a, S: RawData, K, const N: usize> ReverseKernel<'a, S, N> for K
where
    K: IntoKernelWithDilation<'a, S, N>,
{
    fn reverse(self) -> KernelWithDilation<'a, S, N> {
        let mut k = self.into_kernel_with_dilation();
        k.reverse = true;
        k
    }

    fn no_reverse(self) -> KernelWithDilation<'a, S, N> {
        let mut k = self.into_kernel_with_dilation();
        k.reverse = false;
        k
    }
}
