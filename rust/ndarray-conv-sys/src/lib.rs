//! Raw bindings to libndconv: one `extern "C"` declaration per function of
//! include/ndconv.h, the `ndconv_problem` descriptor with the same layout,
//! and the handful of CUDA runtime calls the safe layer needs for device
//! buffers.  Every function returns an `ndconv_status` (`i32`) unless noted;
//! `ndconv_last_error` gives the calling thread's last message.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_void};

// ---- ndconv_dtype
pub const NDCONV_F32: i32 = 0;
pub const NDCONV_F64: i32 = 1;
pub const NDCONV_I32: i32 = 2;
pub const NDCONV_C32: i32 = 3;
pub const NDCONV_C64: i32 = 4;
pub const NDCONV_I64: i32 = 5;
pub const NDCONV_U8: i32 = 6;
pub const NDCONV_I8: i32 = 7;
pub const NDCONV_I16: i32 = 8;
pub const NDCONV_U16: i32 = 9;
pub const NDCONV_U32: i32 = 10;
pub const NDCONV_U64: i32 = 11;

// ---- ndconv_status
pub const NDCONV_OK: i32 = 0;
pub const NDCONV_ERR_DATA_SHAPE: i32 = 1;
pub const NDCONV_ERR_KERNEL_SHAPE: i32 = 2;
pub const NDCONV_ERR_MISMATCH_SHAPE: i32 = 3;
pub const NDCONV_ERR_PAD_OUT_OF_RANGE: i32 = 4;
pub const NDCONV_ERR_UNSUPPORTED: i32 = 5;
pub const NDCONV_ERR_INVALID: i32 = 6;
pub const NDCONV_ERR_CUDA: i32 = 7;
pub const NDCONV_ERR_TIMEOUT: i32 = 8;
pub const NDCONV_ERR_NO_MEMORY: i32 = 9;

// ---- ndconv_conv_mode
pub const NDCONV_MODE_FULL: i32 = 0;
pub const NDCONV_MODE_SAME: i32 = 1;
pub const NDCONV_MODE_VALID: i32 = 2;
pub const NDCONV_MODE_CUSTOM: i32 = 3;
pub const NDCONV_MODE_EXPLICIT: i32 = 4;

// ---- ndconv_border
pub const NDCONV_BORDER_ZEROS: i32 = 0;
pub const NDCONV_BORDER_CONST: i32 = 1;
pub const NDCONV_BORDER_REFLECT: i32 = 2;
pub const NDCONV_BORDER_REPLICATE: i32 = 3;
pub const NDCONV_BORDER_CIRCULAR: i32 = 4;

// ---- ndconv_padding_mode
pub const NDCONV_PAD_ZEROS: i32 = 0;
pub const NDCONV_PAD_CONST: i32 = 1;
pub const NDCONV_PAD_REFLECT: i32 = 2;
pub const NDCONV_PAD_REPLICATE: i32 = 3;
pub const NDCONV_PAD_CIRCULAR: i32 = 4;
pub const NDCONV_PAD_CUSTOM: i32 = 5;
pub const NDCONV_PAD_EXPLICIT: i32 = 6;

// ---- ndconv_algo
pub const NDCONV_ALGO_DIRECT: i32 = 0;
pub const NDCONV_ALGO_FFT: i32 = 1;
pub const NDCONV_ALGO_DIRECT_BF16X3: i32 = 2;
pub const NDCONV_ALGO_FFT_ND: i32 = 3;
pub const NDCONV_ALGO_FFT_RS: i32 = 4;
pub const NDCONV_ALGO_FFT_ND_POW2: i32 = 5;
pub const NDCONV_ALGO_FFT_RS_POW2: i32 = 6;

// ---- ndconv_tune_knob
pub const NDCONV_TUNE_SW_TY: i32 = 0;
pub const NDCONV_TUNE_MAC_ROWS: i32 = 1;
pub const NDCONV_TUNE_ROW_THREADS: i32 = 2;
pub const NDCONV_TUNE_BF16X3_BN: i32 = 3;
pub const NDCONV_TUNE_SW_RY: i32 = 4;

pub const NDCONV_MAX_RANK: usize = 3;

/// `struct ndconv_problem` of include/ndconv.h (same field order and types).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct ndconv_problem {
    pub dtype: i32,
    pub rank: i32,
    pub data_shape: [i64; 3],
    pub kernel_shape: [i64; 3],
    pub dilation: [i64; 3],
    pub reverse: i32,
    pub conv_mode: i32,
    pub mode_padding: [[i64; 2]; 3],
    pub mode_strides: [i64; 3],
    pub padding_mode: i32,
    pub border_kind: [[i32; 2]; 3],
    pub border_value: [[[f64; 2]; 2]; 3],
    pub const_value: [f64; 2],
    pub data_strides: [i64; 3],
    pub kernel_strides: [i64; 3],
}

#[repr(C)]
pub struct ndconv_fft_processor {
    _private: [u8; 0],
}
#[repr(C)]
pub struct ndconv_batch_plan {
    _private: [u8; 0],
}
#[repr(C)]
pub struct ndconv_mlp {
    _private: [u8; 0],
}

#[link(name = "ndconv")]
extern "C" {
    pub fn ndconv_output_shape(p: *const ndconv_problem, algo: i32, out_shape: *mut i64) -> i32;
    pub fn ndconv_padded_host(p: *const ndconv_problem, x: *const f64, nc: i32, out: *mut f64) -> i32;
    pub fn ndconv_conv(p: *const ndconv_problem, data: *const c_void, kernel: *const c_void, out: *mut c_void,
                       stream: *mut c_void) -> i32;
    pub fn ndconv_conv_fft(p: *const ndconv_problem, data: *const c_void, kernel: *const c_void,
                           out: *mut c_void, proc_: *mut ndconv_fft_processor, stream: *mut c_void) -> i32;
    pub fn ndconv_conv_algo(p: *const ndconv_problem, algo: i32, data: *const c_void, kernel: *const c_void,
                            out: *mut c_void, stream: *mut c_void) -> i32;
    pub fn ndconv_conv_batch_host(p: *const ndconv_problem, algo: i32, n: i64, data: *const *const c_void,
                                  kernel: *const *const c_void, out: *const *mut c_void,
                                  proc_: *mut ndconv_fft_processor, stream: *mut c_void) -> i32;
    pub fn ndconv_conv_bf16x3(p: *const ndconv_problem, data: *const c_void, kernel: *const c_void,
                              out: *mut c_void, stream: *mut c_void) -> i32;
    pub fn ndconv_conv_bf16x3_batch(p: *const ndconv_problem, n: i64, data: *const *const c_void,
                                    kernel: *const *const c_void, out: *const *mut c_void,
                                    stream: *mut c_void) -> i32;
    /// `out` holds 18 values (the tile plan, then a folded row's S and R).
    pub fn ndconv_bf16x3_plan(p: *const ndconv_problem, out: *mut i64) -> i32;
    pub fn ndconv_bf16x3_status(stream: *mut c_void) -> i32;
    pub fn ndconv_conv_batch(p: *const ndconv_problem, n: i64, data: *const *const c_void,
                             kernel: *const *const c_void, out: *const *mut c_void, stream: *mut c_void) -> i32;
    pub fn ndconv_conv_fft_batch(p: *const ndconv_problem, n: i64, data: *const *const c_void,
                                 kernel: *const *const c_void, out: *const *mut c_void,
                                 proc_: *mut ndconv_fft_processor, stream: *mut c_void) -> i32;
    pub fn ndconv_batch_create(problems: *const ndconv_problem, n: i64, algo: *const i32,
                               data: *const *const c_void, kernel: *const *const c_void,
                               out: *const *mut c_void, plan: *mut *mut ndconv_batch_plan) -> i32;
    pub fn ndconv_batch_run(plan: *mut ndconv_batch_plan, use_graph: i32, stream: *mut c_void) -> i32;
    pub fn ndconv_batch_run_plain(plan: *mut ndconv_batch_plan, stream: *mut c_void) -> i32;
    pub fn ndconv_batch_status(plan: *mut ndconv_batch_plan, stream: *mut c_void) -> i32;
    pub fn ndconv_batch_set_wait_limit(plan: *mut ndconv_batch_plan, polls: i64) -> i32;
    pub fn ndconv_batch_stall_one_wait(plan: *mut ndconv_batch_plan, enable: i32) -> i32;
    pub fn ndconv_batch_info(plan: *const ndconv_batch_plan, info: *mut i64) -> i32;
    pub fn ndconv_batch_destroy(plan: *mut ndconv_batch_plan) -> i32;
    pub fn ndconv_conv_fft_noalloc(p: *const ndconv_problem, data: *const c_void, kernel: *const c_void,
                                   out: *mut c_void, stream: *mut c_void) -> i32;
    pub fn ndconv_fft_processor_create(dtype: i32, out: *mut *mut ndconv_fft_processor) -> i32;
    pub fn ndconv_fft_processor_destroy(proc_: *mut ndconv_fft_processor) -> i32;
    pub fn ndconv_fft_processor_bake(proc_: *mut ndconv_fft_processor, p: *const ndconv_problem,
                                     kernel: *const c_void, stream: *mut c_void) -> i32;
    pub fn ndconv_fft_forward(proc_: *mut ndconv_fft_processor, rank: i32, shape: *const i64, input: *const c_void,
                              out: *mut c_void, out_shape: *mut i64, stream: *mut c_void) -> i32;
    pub fn ndconv_fft_backward(proc_: *mut ndconv_fft_processor, rank: i32, shape: *const i64,
                               input: *const c_void, out: *mut c_void, out_shape: *mut i64,
                               stream: *mut c_void) -> i32;
    /// Kernels this library launched in the process so far.
    pub fn ndconv_kernel_launches() -> u64;
    pub fn ndconv_plan_info(p: *const ndconv_problem, out: *mut f64) -> i32;
    /// Thread-local tile / plan knob for the autotuner (0: the library chooses).
    pub fn ndconv_set_tuning(knob: i32, value: i32) -> i32;
    /// The knob's current value (not a status).
    pub fn ndconv_get_tuning(knob: i32) -> i32;
    /// The calling thread's last error message (never null).
    pub fn ndconv_last_error() -> *const c_char;
    pub fn ndconv_version() -> *const c_char;
    pub fn ndconv_mlp_create(n_in: i32, n_hidden: i32, n_out: i32, seed: u64, out: *mut *mut ndconv_mlp) -> i32;
    pub fn ndconv_mlp_destroy(net: *mut ndconv_mlp) -> i32;
    /// Number of parameters of the network (not a status).
    pub fn ndconv_mlp_param_count(net: *const ndconv_mlp) -> i64;
    pub fn ndconv_mlp_params(net: *mut ndconv_mlp, host: *mut f32, n: i64, set: i32) -> i32;
    pub fn ndconv_mlp_forward(net: *mut ndconv_mlp, x: *const f32, n: i64, y: *mut f32, stream: *mut c_void) -> i32;
    pub fn ndconv_mlp_gradient(net: *mut ndconv_mlp, x: *const f32, target: *const f32, mask: *const f32, n: i64,
                               grad: *mut f32, loss: *mut f32, stream: *mut c_void) -> i32;
    pub fn ndconv_mlp_train(net: *mut ndconv_mlp, x: *const f32, target: *const f32, mask: *const f32, n: i64,
                            epochs: i32, batch: i32, lr: f32, seed: u64, final_loss: *mut f32,
                            stream: *mut c_void) -> i32;
}

/// The CUDA runtime calls the safe layer uses for its device buffers.
pub mod cuda {
    use std::os::raw::c_void;

    pub const MEMCPY_HOST_TO_DEVICE: i32 = 1;
    pub const MEMCPY_DEVICE_TO_HOST: i32 = 2;

    #[link(name = "cudart")]
    extern "C" {
        pub fn cudaMalloc(ptr: *mut *mut c_void, bytes: usize) -> i32;
        pub fn cudaFree(ptr: *mut c_void) -> i32;
        pub fn cudaMemcpy(dst: *mut c_void, src: *const c_void, bytes: usize, kind: i32) -> i32;
        pub fn cudaStreamSynchronize(stream: *mut c_void) -> i32;
    }
}
