//! The device side of the shim: which element types the library runs, the
//! `ndconv_problem` descriptor built from the crate's arguments, device
//! buffers, and the mapping of status codes to `Error<N>` (or a panic where
//! the original panics or the device itself failed).
use std::ffi::CStr;
use std::os::raw::c_void;

use ndarray::{Array, ArrayBase, Data, Dim, Ix};
use ndarray_conv_sys as sys;
use num::Complex;

use crate::{BorderType, ConvMode, Error, KernelWithDilation, PaddingMode};

/// Element types with a device implementation: f32, f64, Complex<f32>,
/// Complex<f64> and the 8- to 64-bit integers (wrapping sums; integers other
/// than i32 run `conv` one call at a time, and integer FFT convolution is
/// refused as upstream documents it broken).  The original accepts any
/// `NumAssign + Copy` type.
pub trait DeviceElem: num::traits::NumAssign + Copy + 'static {
    /// `ndconv_dtype`
    const DTYPE: i32;
    /// (re, im) of a border constant
    fn parts(self) -> [f64; 2];
}

impl DeviceElem for f32 {
    const DTYPE: i32 = sys::NDCONV_F32;
    fn parts(self) -> [f64; 2] {
        [self as f64, 0.0]
    }
}
impl DeviceElem for f64 {
    const DTYPE: i32 = sys::NDCONV_F64;
    fn parts(self) -> [f64; 2] {
        [self, 0.0]
    }
}
impl DeviceElem for i32 {
    const DTYPE: i32 = sys::NDCONV_I32;
    fn parts(self) -> [f64; 2] {
        [self as f64, 0.0]
    }
}
macro_rules! device_int {
    ($($t:ty => $code:ident),*) => {$(
        impl DeviceElem for $t {
            const DTYPE: i32 = sys::$code;
            fn parts(self) -> [f64; 2] {
                [self as f64, 0.0]
            }
        }
    )*};
}
device_int!(i8 => NDCONV_I8, u8 => NDCONV_U8, i16 => NDCONV_I16, u16 => NDCONV_U16, u32 => NDCONV_U32,
            i64 => NDCONV_I64, u64 => NDCONV_U64);

impl DeviceElem for Complex<f32> {
    const DTYPE: i32 = sys::NDCONV_C32;
    fn parts(self) -> [f64; 2] {
        [self.re as f64, self.im as f64]
    }
}
impl DeviceElem for Complex<f64> {
    const DTYPE: i32 = sys::NDCONV_C64;
    fn parts(self) -> [f64; 2] {
        [self.re, self.im]
    }
}

fn border<T: DeviceElem>(b: BorderType<T>) -> (i32, [f64; 2]) {
    match b {
        BorderType::Zeros => (sys::NDCONV_BORDER_ZEROS, [0.0; 2]),
        BorderType::Const(c) => (sys::NDCONV_BORDER_CONST, c.parts()),
        BorderType::Reflect => (sys::NDCONV_BORDER_REFLECT, [0.0; 2]),
        BorderType::Replicate => (sys::NDCONV_BORDER_REPLICATE, [0.0; 2]),
        BorderType::Circular => (sys::NDCONV_BORDER_CIRCULAR, [0.0; 2]),
    }
}

/// The problem descriptor for contiguous data of shape `data_shape` and the
/// kernel (contiguous after the caller's copy) with its dilation and flip.
pub(crate) fn problem<T: DeviceElem, S: Data<Elem = T>, const N: usize>(
    data_shape: &[usize],
    kernel: &KernelWithDilation<'_, S, N>,
    conv_mode: ConvMode<N>,
    padding_mode: PaddingMode<N, T>,
) -> sys::ndconv_problem {
    assert!(N >= 1 && N <= sys::NDCONV_MAX_RANK, "ndarray-conv (GPU): ranks 1 to 3 only");
    let mut p = sys::ndconv_problem { dtype: T::DTYPE, rank: N as i32, ..Default::default() };
    let kshape = kernel.kernel.shape();
    for i in 0..N {
        p.data_shape[i] = data_shape[i] as i64;
        p.kernel_shape[i] = kshape[i] as i64;
        p.dilation[i] = kernel.dilation[i] as i64;
        p.mode_strides[i] = 1;
    }
    p.reverse = kernel.reverse as i32;
    match conv_mode {
        ConvMode::Full => p.conv_mode = sys::NDCONV_MODE_FULL,
        ConvMode::Same => p.conv_mode = sys::NDCONV_MODE_SAME,
        ConvMode::Valid => p.conv_mode = sys::NDCONV_MODE_VALID,
        ConvMode::Custom { padding, strides } => {
            p.conv_mode = sys::NDCONV_MODE_CUSTOM;
            for i in 0..N {
                p.mode_padding[i] = [padding[i] as i64; 2];
                p.mode_strides[i] = strides[i] as i64;
            }
        }
        ConvMode::Explicit { padding, strides } => {
            p.conv_mode = sys::NDCONV_MODE_EXPLICIT;
            for i in 0..N {
                p.mode_padding[i] = [padding[i][0] as i64, padding[i][1] as i64];
                p.mode_strides[i] = strides[i] as i64;
            }
        }
    }
    match padding_mode {
        PaddingMode::Zeros => p.padding_mode = sys::NDCONV_PAD_ZEROS,
        PaddingMode::Const(c) => {
            p.padding_mode = sys::NDCONV_PAD_CONST;
            p.const_value = c.parts();
        }
        PaddingMode::Reflect => p.padding_mode = sys::NDCONV_PAD_REFLECT,
        PaddingMode::Replicate => p.padding_mode = sys::NDCONV_PAD_REPLICATE,
        PaddingMode::Circular => p.padding_mode = sys::NDCONV_PAD_CIRCULAR,
        PaddingMode::Custom(b) => {
            p.padding_mode = sys::NDCONV_PAD_CUSTOM;
            for i in 0..N {
                let (kind, v) = border(b[i]);
                p.border_kind[i] = [kind, kind];
                p.border_value[i] = [v, v];
            }
        }
        PaddingMode::Explicit(b) => {
            p.padding_mode = sys::NDCONV_PAD_EXPLICIT;
            for i in 0..N {
                let (k0, v0) = border(b[i][0]);
                let (k1, v1) = border(b[i][1]);
                p.border_kind[i] = [k0, k1];
                p.border_value[i] = [v0, v1];
            }
        }
    }
    p
}

pub(crate) fn last_error() -> String {
    unsafe { CStr::from_ptr(sys::ndconv_last_error()) }.to_string_lossy().into_owned()
}

/// A status that is not a shape error: the original panics there (padding
/// out of range) or the device failed.
pub(crate) fn fail(st: i32) -> ! {
    panic!("ndarray-conv (GPU): status {st}: {}", last_error())
}

/// Status of a host-side check (`ndconv_output_shape`) as the original's
/// `Error<N>`.  `fft` selects the FFT path's report of a zero-size kernel
/// (`DataShape` with the kernel's dimensions).
pub(crate) fn shape_error<const N: usize>(
    st: i32,
    fft: bool,
    data_shape: [usize; N],
    kernel_shape: [usize; N],
    dilation: [usize; N],
    conv_mode: ConvMode<N>,
) -> Error<N> {
    match st {
        sys::NDCONV_ERR_DATA_SHAPE => {
            let kernel_zero = kernel_shape.iter().any(|&k| k == 0) && data_shape.iter().all(|&n| n != 0);
            Error::DataShape(ndarray::Dim(if fft && kernel_zero { kernel_shape } else { data_shape }))
        }
        sys::NDCONV_ERR_KERNEL_SHAPE => Error::KernelShape(ndarray::Dim(kernel_shape)),
        sys::NDCONV_ERR_MISMATCH_SHAPE => {
            let keff: [usize; N] = std::array::from_fn(|i| kernel_shape[i] * dilation[i] - dilation[i] + 1);
            Error::MismatchShape(conv_mode, keff)
        }
        _ => fail(st),
    }
}

/// A device allocation freed on drop.
pub(crate) struct DeviceBuffer {
    pub(crate) ptr: *mut c_void,
}

impl DeviceBuffer {
    pub(crate) fn alloc(bytes: usize) -> DeviceBuffer {
        let mut ptr = std::ptr::null_mut();
        let e = unsafe { sys::cuda::cudaMalloc(&mut ptr, bytes.max(1)) };
        if e != 0 {
            panic!("ndarray-conv (GPU): cudaMalloc of {bytes} bytes failed ({e})");
        }
        DeviceBuffer { ptr }
    }

    pub(crate) fn upload<T: Copy>(host: &[T]) -> DeviceBuffer {
        let bytes = std::mem::size_of_val(host);
        let b = DeviceBuffer::alloc(bytes);
        let e = unsafe {
            sys::cuda::cudaMemcpy(b.ptr, host.as_ptr() as *const c_void, bytes, sys::cuda::MEMCPY_HOST_TO_DEVICE)
        };
        if e != 0 {
            panic!("ndarray-conv (GPU): host-to-device copy failed ({e})");
        }
        b
    }

    pub(crate) fn download<T: Copy>(&self, host: &mut [T]) {
        let bytes = std::mem::size_of_val(host);
        let e = unsafe {
            sys::cuda::cudaMemcpy(host.as_mut_ptr() as *mut c_void, self.ptr, bytes, sys::cuda::MEMCPY_DEVICE_TO_HOST)
        };
        if e != 0 {
            panic!("ndarray-conv (GPU): device-to-host copy failed ({e})");
        }
    }
}

impl Drop for DeviceBuffer {
    fn drop(&mut self) {
        unsafe {
            sys::cuda::cudaFree(self.ptr);
        }
    }
}

/// One convolution: `ndconv_output_shape` checks the arguments in the
/// original's order for the chosen path, then the data and kernel go to the
/// device, `call(problem, x, k, y)` runs the entry point on the default
/// stream, and the output comes back as a new array.
pub(crate) fn convolve<T, S, SK, const N: usize>(
    fft: bool,
    data: &ArrayBase<S, Dim<[Ix; N]>>,
    kernel: KernelWithDilation<'_, SK, N>,
    conv_mode: ConvMode<N>,
    padding_mode: PaddingMode<N, T>,
    call: impl FnOnce(&sys::ndconv_problem, *const c_void, *const c_void, *mut c_void) -> i32,
) -> Result<Array<T, Dim<[Ix; N]>>, Error<N>>
where
    T: DeviceElem,
    S: Data<Elem = T>,
    SK: Data<Elem = T>,
    Dim<[Ix; N]>: ndarray::Dimension,
    [Ix; N]: ndarray::IntoDimension<Dim = Dim<[Ix; N]>>,
{
    let dshape: [usize; N] = std::array::from_fn(|i| data.shape()[i]);
    let kshape: [usize; N] = std::array::from_fn(|i| kernel.kernel.shape()[i]);
    let p = problem(&dshape, &kernel, conv_mode, padding_mode);
    let mut osh = [0i64; 3];
    let st = unsafe { sys::ndconv_output_shape(&p, fft as i32, osh.as_mut_ptr()) };
    if st != sys::NDCONV_OK {
        return Err(shape_error(st, fft, dshape, kshape, kernel.dilation, conv_mode));
    }
    let oshape: [usize; N] = std::array::from_fn(|i| osh[i] as usize);
    let x = data.as_standard_layout();
    let k = kernel.kernel.as_standard_layout();
    let dx = DeviceBuffer::upload(x.as_slice().expect("standard layout"));
    let dk = DeviceBuffer::upload(k.as_slice().expect("standard layout"));
    let mut y = Array::<T, Dim<[Ix; N]>>::zeros(oshape);
    let dy = DeviceBuffer::alloc(std::mem::size_of::<T>() * y.len());
    let st = call(&p, dx.ptr, dk.ptr, dy.ptr);
    if st != sys::NDCONV_OK {
        fail(st);
    }
    let e = unsafe { sys::cuda::cudaStreamSynchronize(std::ptr::null_mut()) };
    if e != 0 {
        panic!("ndarray-conv (GPU): the convolution failed on the device ({e})");
    }
    dy.download(y.as_slice_mut().expect("new array is contiguous"));
    Ok(y)
}
