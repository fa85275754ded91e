//! `ConvFFTExt` (conv_fft, conv_fft_with_processor, conv_fft_par) and the FFT
//! processor (`Processor`, `GetProcessor`, `get_fft_processor`), as in the
//! original's src/conv_fft/mod.rs and src/conv_fft/processor/mod.rs, run by
//! `ndconv_conv_fft` and `ndconv_fft_forward` / `ndconv_fft_backward`.  The
//! processor's spectrum layout is the original's (axes rotated right after
//! each pass), so `backward(forward(x))` round-trips the same way.
use std::marker::PhantomData;

use ndarray::{Array, ArrayBase, Data, DataMut, Dim, IntoDimension, Ix, RawData, RemoveAxis};
use ndarray_conv_sys as sys;
use num::Complex;

use crate::device::{convolve, fail, DeviceBuffer, DeviceElem};
use crate::{ConvMode, Error, IntoKernelWithDilation, PaddingMode};

/// Real scalar types of the FFT path: f32 and f64 (the original takes any
/// rustfft `FftNum`; its integer FFT is documented as broken there).
pub trait FftNum: DeviceElem + num::Float {}
impl FftNum for f32 {}
impl FftNum for f64 {}

pub trait Processor<T: FftNum, InElem: GetProcessor<T, InElem>> {
    /// N-d forward transform in the original's rotated layout.  `parallel`
    /// is accepted and ignored: the transform always runs on the GPU.
    fn forward<S: DataMut<Elem = InElem>, const N: usize>(
        &mut self,
        input: &mut ArrayBase<S, Dim<[Ix; N]>>,
        parallel: bool,
    ) -> Array<Complex<T>, Dim<[Ix; N]>>
    where
        Dim<[Ix; N]>: RemoveAxis,
        [Ix; N]: IntoDimension<Dim = Dim<[Ix; N]>>;

    /// Inverse of `forward`, divided by the element count.
    fn backward<const N: usize>(
        &mut self,
        input: &mut Array<Complex<T>, Dim<[Ix; N]>>,
        parallel: bool,
    ) -> Array<InElem, Dim<[Ix; N]>>
    where
        Dim<[Ix; N]>: RemoveAxis,
        [Ix; N]: IntoDimension<Dim = Dim<[Ix; N]>>;

    /// The library processor behind this one, reused by
    /// conv_fft_with_processor (null: none, the call then plans afresh).
    #[doc(hidden)]
    fn device_handle(&mut self) -> *mut sys::ndconv_fft_processor {
        std::ptr::null_mut()
    }
}

pub trait GetProcessor<T: FftNum, InElem>: DeviceElem
where
    InElem: GetProcessor<T, InElem>,
{
    fn get_processor() -> impl Processor<T, InElem>;
}

impl<T: FftNum> GetProcessor<T, T> for T {
    fn get_processor() -> impl Processor<T, T> {
        FftProcessor::<T, T>::new()
    }
}

impl<T: FftNum> GetProcessor<T, Complex<T>> for Complex<T>
where
    Complex<T>: DeviceElem,
{
    fn get_processor() -> impl Processor<T, Complex<T>> {
        FftProcessor::<T, Complex<T>>::new()
    }
}

/// `get_fft_processor::<T, InElem>()` of the original.
pub fn get_processor<T: FftNum, InElem: GetProcessor<T, InElem>>() -> impl Processor<T, InElem> {
    InElem::get_processor()
}

/// The library's FFT processor (`ndconv_fft_processor`): cached plans,
/// twiddle tables and a grow-only workspace on the current device.
pub struct FftProcessor<T: FftNum, InElem> {
    handle: *mut sys::ndconv_fft_processor,
    _types: PhantomData<(T, InElem)>,
}

// the library processor is used by one thread at a time (`&mut self`), as
// the original's processor under rayon
unsafe impl<T: FftNum, InElem> Send for FftProcessor<T, InElem> {}

impl<T: FftNum, InElem: DeviceElem> FftProcessor<T, InElem> {
    pub fn new() -> Self {
        let mut handle = std::ptr::null_mut();
        let st = unsafe { sys::ndconv_fft_processor_create(InElem::DTYPE, &mut handle) };
        if st != sys::NDCONV_OK {
            fail(st);
        }
        FftProcessor { handle, _types: PhantomData }
    }
}

impl<T: FftNum, InElem: DeviceElem> Default for FftProcessor<T, InElem> {
    fn default() -> Self {
        Self::new()
    }
}

impl<T: FftNum, InElem> Drop for FftProcessor<T, InElem> {
    fn drop(&mut self) {
        unsafe {
            sys::ndconv_fft_processor_destroy(self.handle);
        }
    }
}

fn sync() {
    let e = unsafe { sys::cuda::cudaStreamSynchronize(std::ptr::null_mut()) };
    if e != 0 {
        panic!("ndarray-conv (GPU): FFT processor failed on the device ({e})");
    }
}

impl<T: FftNum, InElem: GetProcessor<T, InElem>> Processor<T, InElem> for FftProcessor<T, InElem> {
    fn forward<S: DataMut<Elem = InElem>, const N: usize>(
        &mut self,
        input: &mut ArrayBase<S, Dim<[Ix; N]>>,
        _parallel: bool,
    ) -> Array<Complex<T>, Dim<[Ix; N]>>
    where
        Dim<[Ix; N]>: RemoveAxis,
        [Ix; N]: IntoDimension<Dim = Dim<[Ix; N]>>,
    {
        let mut shape = [1i64; 3];
        for i in 0..N {
            shape[i] = input.shape()[i] as i64;
        }
        let null = std::ptr::null_mut();
        let mut osh = [0i64; 3];
        let st = unsafe {
            sys::ndconv_fft_forward(self.handle, N as i32, shape.as_ptr(), std::ptr::null(), null, osh.as_mut_ptr(), null)
        };
        if st != sys::NDCONV_OK {
            fail(st);
        }
        let x = input.as_standard_layout();
        let dx = DeviceBuffer::upload(x.as_slice().expect("standard layout"));
        let oshape: [usize; N] = std::array::from_fn(|i| osh[i] as usize);
        let mut out = Array::<Complex<T>, Dim<[Ix; N]>>::zeros(oshape);
        let dy = DeviceBuffer::alloc(std::mem::size_of::<Complex<T>>() * out.len());
        let st = unsafe { sys::ndconv_fft_forward(self.handle, N as i32, shape.as_ptr(), dx.ptr, dy.ptr, osh.as_mut_ptr(), null) };
        if st != sys::NDCONV_OK {
            fail(st);
        }
        sync();
        dy.download(out.as_slice_mut().expect("new array is contiguous"));
        out
    }

    fn backward<const N: usize>(
        &mut self,
        input: &mut Array<Complex<T>, Dim<[Ix; N]>>,
        _parallel: bool,
    ) -> Array<InElem, Dim<[Ix; N]>>
    where
        Dim<[Ix; N]>: RemoveAxis,
        [Ix; N]: IntoDimension<Dim = Dim<[Ix; N]>>,
    {
        let mut shape = [1i64; 3];
        for i in 0..N {
            shape[i] = input.shape()[i] as i64;
        }
        let null = std::ptr::null_mut();
        let mut osh = [0i64; 3];
        let st = unsafe {
            sys::ndconv_fft_backward(self.handle, N as i32, shape.as_ptr(), std::ptr::null(), null, osh.as_mut_ptr(), null)
        };
        if st != sys::NDCONV_OK {
            fail(st);
        }
        let s = input.as_standard_layout();
        let ds = DeviceBuffer::upload(s.as_slice().expect("standard layout"));
        let oshape: [usize; N] = std::array::from_fn(|i| osh[i] as usize);
        let mut out = Array::<InElem, Dim<[Ix; N]>>::zeros(oshape);
        let dy = DeviceBuffer::alloc(std::mem::size_of::<InElem>() * out.len());
        let st = unsafe { sys::ndconv_fft_backward(self.handle, N as i32, shape.as_ptr(), ds.ptr, dy.ptr, osh.as_mut_ptr(), null) };
        if st != sys::NDCONV_OK {
            fail(st);
        }
        sync();
        dy.download(out.as_slice_mut().expect("new array is contiguous"));
        out
    }

    fn device_handle(&mut self) -> *mut sys::ndconv_fft_processor {
        self.handle
    }
}

pub trait ConvFFTExt<'a, T, InElem, S, SK, const N: usize>
where
    T: num::traits::NumAssign + Copy + FftNum,
    InElem: GetProcessor<T, InElem> + Copy + num::traits::NumAssign,
    S: RawData,
    SK: RawData,
{
    fn conv_fft(
        &self,
        kernel: impl IntoKernelWithDilation<'a, SK, N>,
        conv_mode: ConvMode<N>,
        padding_mode: PaddingMode<N, InElem>,
    ) -> Result<Array<InElem, Dim<[Ix; N]>>, Error<N>>;

    /// conv_fft reusing the processor's cached plans and workspace (and its
    /// baked kernel spectrum, if the library processor holds one for this
    /// geometry and kernel).
    fn conv_fft_with_processor(
        &self,
        kernel: impl IntoKernelWithDilation<'a, SK, N>,
        conv_mode: ConvMode<N>,
        padding_mode: PaddingMode<N, InElem>,
        fft_processor: &mut impl Processor<T, InElem>,
    ) -> Result<Array<InElem, Dim<[Ix; N]>>, Error<N>>;

    /// The original's rayon version; on the GPU every call is parallel, so
    /// this is conv_fft.
    #[cfg(feature = "rayon")]
    fn conv_fft_par(
        &self,
        kernel: impl IntoKernelWithDilation<'a, SK, N>,
        conv_mode: ConvMode<N>,
        padding_mode: PaddingMode<N, InElem>,
    ) -> Result<Array<InElem, Dim<[Ix; N]>>, Error<N>>;
}

impl<'a, T, InElem, S, SK, const N: usize> ConvFFTExt<'a, T, InElem, S, SK, N> for ArrayBase<S, Dim<[Ix; N]>>
where
    T: FftNum,
    InElem: GetProcessor<T, InElem>,
    S: Data<Elem = InElem> + 'a,
    SK: Data<Elem = InElem> + 'a,
    Dim<[Ix; N]>: ndarray::Dimension,
    [Ix; N]: IntoDimension<Dim = Dim<[Ix; N]>>,
{
    fn conv_fft(
        &self,
        kernel: impl IntoKernelWithDilation<'a, SK, N>,
        conv_mode: ConvMode<N>,
        padding_mode: PaddingMode<N, InElem>,
    ) -> Result<Array<InElem, Dim<[Ix; N]>>, Error<N>> {
        let kernel = kernel.into_kernel_with_dilation();
        convolve(true, self, kernel, conv_mode, padding_mode, |p, x, k, y| unsafe {
            sys::ndconv_conv_fft(p, x, k, y, std::ptr::null_mut(), std::ptr::null_mut())
        })
    }

    fn conv_fft_with_processor(
        &self,
        kernel: impl IntoKernelWithDilation<'a, SK, N>,
        conv_mode: ConvMode<N>,
        padding_mode: PaddingMode<N, InElem>,
        fft_processor: &mut impl Processor<T, InElem>,
    ) -> Result<Array<InElem, Dim<[Ix; N]>>, Error<N>> {
        let kernel = kernel.into_kernel_with_dilation();
        let handle = fft_processor.device_handle();
        convolve(true, self, kernel, conv_mode, padding_mode, |p, x, k, y| unsafe {
            sys::ndconv_conv_fft(p, x, k, y, handle, std::ptr::null_mut())
        })
    }

    #[cfg(feature = "rayon")]
    fn conv_fft_par(
        &self,
        kernel: impl IntoKernelWithDilation<'a, SK, N>,
        conv_mode: ConvMode<N>,
        padding_mode: PaddingMode<N, InElem>,
    ) -> Result<Array<InElem, Dim<[Ix; N]>>, Error<N>> {
        self.conv_fft(kernel, conv_mode, padding_mode)
    }
}
