//! `ndarray-conv` on a GB300: the crate's public API (`ConvExt::conv`,
//! `ConvFFTExt::conv_fft` / `conv_fft_with_processor` / `conv_fft_par`,
//! `ConvMode`, `PaddingMode`, `BorderType`, `with_dilation`, `no_reverse`,
//! `Complex<T>`, `GetProcessor`) with every convolution run by the sm_103a
//! kernels of libndconv through `ndarray-conv-sys`.  Arrays are copied to
//! device buffers, convolved there, and the result comes back as a new
//! owned `Array`, as the original returns.
//!
//! Differences a caller can see:
//! * element types: f32, f64, i32 (direct `conv` only), `Complex<f32>` and
//!   `Complex<f64>` (the `DeviceElem` bound); ranks 1 to 3;
//! * failures of the device itself (CUDA errors, a bounded device wait that
//!   ran out) panic with the library's message, like the padding cases where
//!   the original panics; shape errors are the same `Error<N>` values.
mod conv;
mod conv_fft;
mod device;
mod dilation;
mod tensor;

pub use conv::ConvExt;
pub use conv_fft::{get_processor as get_fft_processor, ConvFFTExt, FftNum, FftProcessor, GetProcessor, Processor};
pub use device::DeviceElem;
pub use dilation::{IntoDilation, IntoKernelWithDilation, KernelWithDilation, ReverseKernel, WithDilation};
pub use tensor::{ConvTensorExt, TensorElem};

/// How the output size is determined (the original's `ConvMode<N>`).
#[derive(Debug, Clone, Copy)]
pub enum ConvMode<const N: usize> {
    /// every position where kernel and input overlap at least partially
    Full,
    /// the input's size
    Same,
    /// only positions where the kernel lies inside the input
    Valid,
    /// the same padding on both sides of each axis, and strides
    Custom { padding: [usize; N], strides: [usize; N] },
    /// padding per side of each axis, and strides
    Explicit { padding: [[usize; 2]; N], strides: [usize; N] },
}

/// How borders are filled (the original's `PaddingMode<N, T>`).
#[derive(Debug, Clone, Copy)]
pub enum PaddingMode<const N: usize, T: num::traits::NumAssign + Copy> {
    Zeros,
    Const(T),
    Reflect,
    Replicate,
    Circular,
    /// one `BorderType` per axis, both sides
    Custom([BorderType<T>; N]),
    /// one `BorderType` per side of each axis
    Explicit([[BorderType<T>; 2]; N]),
}

/// One side's fill (the original's `BorderType<T>`).
#[derive(Debug, Clone, Copy)]
pub enum BorderType<T: num::traits::NumAssign + Copy> {
    Zeros,
    Const(T),
    Reflect,
    Replicate,
    Circular,
}

/// Shape errors, as the original reports them.
#[derive(thiserror::Error, Debug)]
pub enum Error<const N: usize> {
    #[error("Data shape shouldn't have ZERO. {0:?}")]
    DataShape(ndarray::Dim<[ndarray::Ix; N]>),
    #[error("Kernel shape shouldn't have ZERO. {0:?}")]
    KernelShape(ndarray::Dim<[ndarray::Ix; N]>),
    #[error("ConvMode {0:?} does not match KernelWithDilation Size {1:?}")]
    MismatchShape(ConvMode<N>, [ndarray::Ix; N]),
}
