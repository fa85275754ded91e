/*
 * ndconv -- C ABI of the GB300 (sm_103a) convolution library.
 *
 * Drop-in boundary for the convolution hot path of the ndarray-conv crate
 * (v0.6.1).  Every entry point names the reference interface it replaces.
 * Plain pointers and sizes only: device pointers for data, kernel and
 * output; `stream` is a cudaStream_t passed as void* (NULL = legacy default
 * stream).  All calls are asynchronous on `stream` unless stated.
 *
 * Arrays are row-major N-d views (N = rank, 1..3) with ELEMENT strides
 * (0 in every slot = contiguous).  Complex elements are interleaved re, im.
 * Outputs are always written contiguous row-major.
 *
 * Status codes mirror the reference's Result<_, Error<N>>
 * (src/lib.rs:148-159); the reference's panics become
 * NDCONV_ERR_PAD_OUT_OF_RANGE.
 */
#ifndef NDCONV_H
#define NDCONV_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NDCONV_MAX_RANK 3

/* element type (InElem / T of the reference traits).  The crate's ConvExt
 * is generic over any T: NumAssign + Copy and any rank N
 * (src/conv/mod.rs:78-83,118-124); its own tests pad u8 arrays
 * (src/padding/mod.rs:621-624).  This library runs ranks 1..NDCONV_MAX_RANK
 * and the element types below; any other code and any rank above 3 get
 * NDCONV_ERR_UNSUPPORTED (there is no CPU fallback).  Integers use wrapping
 * arithmetic, as release-mode Rust does (the sum of products modulo 2^bits),
 * and take the direct path only (integer FFT convolution is documented
 * broken upstream, src/conv_fft/processor/mod.rs:46-59).  i32 runs every
 * direct entry point (single, batch, host batch, batch plans); the other
 * integer types run ndconv_conv and ndconv_conv_algo(NDCONV_ALGO_DIRECT)
 * (and ndconv_output_shape) and are refused by the rest.  8- and 16-bit
 * data are widened to 32 bits on the device (stream-ordered scratch), summed
 * by the 32-bit kernels and truncated: the low bits of a wrapping sum depend
 * only on the low bits of its terms, so results are the element type's own
 * wrapping sums.  Unsigned types share their signed twin's kernels bit for
 * bit. */
typedef enum {
    NDCONV_F32 = 0,
    NDCONV_F64 = 1,
    NDCONV_I32 = 2, /* direct conv only, wrapping arithmetic (release-mode Rust) */
    NDCONV_C32 = 3, /* num_complex::Complex<f32> */
    NDCONV_C64 = 4,
    NDCONV_I64 = 5, /* the integer types from here on: ndconv_conv only */
    NDCONV_U8 = 6,
    NDCONV_I8 = 7,
    NDCONV_I16 = 8,
    NDCONV_U16 = 9,
    NDCONV_U32 = 10,
    NDCONV_U64 = 11
} ndconv_dtype;

typedef enum {
    NDCONV_OK = 0,
    NDCONV_ERR_DATA_SHAPE = 1,      /* Error::DataShape (also zero-size kernel on the FFT path, src/conv_fft/mod.rs:211-212) */
    NDCONV_ERR_KERNEL_SHAPE = 2,    /* Error::KernelShape (direct path, src/conv/mod.rs:142-144) */
    NDCONV_ERR_MISMATCH_SHAPE = 3,  /* Error::MismatchShape (src/conv/mod.rs:152-158, src/conv_fft/mod.rs:220-227) */
    NDCONV_ERR_PAD_OUT_OF_RANGE = 4,/* the reference panics: reflect index out of range (src/padding/half_dim.rs:192-210,233-258) */
    NDCONV_ERR_UNSUPPORTED = 5,     /* e.g. integer FFT (documented broken upstream, src/conv_fft/processor/mod.rs:46-59) */
    NDCONV_ERR_INVALID = 6,         /* bad argument (rank, zero stride/dilation, null pointer) */
    NDCONV_ERR_CUDA = 7,
    NDCONV_ERR_TIMEOUT = 8,         /* a bounded device-side wait ran out */
    NDCONV_ERR_NO_MEMORY = 9
} ndconv_status;

/* ConvMode<N> (src/lib.rs:81-105) */
typedef enum {
    NDCONV_MODE_FULL = 0,
    NDCONV_MODE_SAME = 1,
    NDCONV_MODE_VALID = 2,
    NDCONV_MODE_CUSTOM = 3,   /* padding[i][0] on both sides, strides[i] */
    NDCONV_MODE_EXPLICIT = 4  /* padding[i][0..2], strides[i] */
} ndconv_conv_mode;

/* BorderType<T> (src/lib.rs:131-143) */
typedef enum {
    NDCONV_BORDER_ZEROS = 0,
    NDCONV_BORDER_CONST = 1,
    NDCONV_BORDER_REFLECT = 2,
    NDCONV_BORDER_REPLICATE = 3,
    NDCONV_BORDER_CIRCULAR = 4
} ndconv_border;

/* PaddingMode<N, T> (src/lib.rs:111-127) */
typedef enum {
    NDCONV_PAD_ZEROS = 0,
    NDCONV_PAD_CONST = 1,
    NDCONV_PAD_REFLECT = 2,
    NDCONV_PAD_REPLICATE = 3,
    NDCONV_PAD_CIRCULAR = 4,
    NDCONV_PAD_CUSTOM = 5,    /* border_kind[i][0] per axis, both sides */
    NDCONV_PAD_EXPLICIT = 6   /* border_kind[i][0] front, [i][1] back */
} ndconv_padding_mode;

/*
 * One convolution problem: data view, kernel view with dilation and the
 * reverse flag (KernelWithDilation, src/dilation/mod.rs:8-12), ConvMode and
 * PaddingMode.
 */
typedef struct ndconv_problem {
    int32_t dtype;                 /* ndconv_dtype */
    int32_t rank;                  /* 1..3 */
    int64_t data_shape[3];
    int64_t kernel_shape[3];
    int64_t dilation[3];           /* >= 1 (with_dilation, src/dilation/mod.rs:103-126) */
    int32_t reverse;               /* 1 = convolution (default), 0 = no_reverse() */
    int32_t conv_mode;             /* ndconv_conv_mode */
    int64_t mode_padding[3][2];
    int64_t mode_strides[3];
    int32_t padding_mode;          /* ndconv_padding_mode */
    int32_t border_kind[3][2];     /* ndconv_border */
    double border_value[3][2][2];  /* BorderType::Const(c): (re, im) per axis and side */
    double const_value[2];         /* PaddingMode::Const(c): (re, im) */
    int64_t data_strides[3];       /* element strides, all 0 = contiguous */
    int64_t kernel_strides[3];     /* element strides, all 0 = contiguous */
} ndconv_problem;

typedef struct ndconv_fft_processor ndconv_fft_processor;
typedef struct ndconv_batch_plan ndconv_batch_plan;

/* Output shape and argument checks, host only (no device work).
 * algo: 0 = direct (ConvExt::conv), 1 = FFT (ConvFFTExt::conv_fft); the two
 * paths report zero-size kernels and padding panics in the reference's
 * different orders. */
int ndconv_output_shape(const ndconv_problem *p, int32_t algo, int64_t out_shape[3]);

/* The padded array that ConvExt::conv convolves, as the crate's
 * PaddingExt::padding materialises it (src/padding/mod.rs:84-452, dim.rs,
 * half_dim.rs), from the closed-form border map that every kernel of this
 * library evaluates in its loads instead of storing a padded copy.  Host
 * only (no device work).  x: the problem's data on the host as f64 (nc = 1)
 * or (re, im) pairs (nc = 2), in its element strides; out: the padded
 * extents (input + both pads per axis), contiguous.  Padding that makes
 * the crate panic is reported as NDCONV_ERR_PAD_OUT_OF_RANGE. */
int ndconv_padded_host(const ndconv_problem *p, const double *x, int32_t nc, double *out);

/* ConvExt::conv (src/conv/mod.rs:78-116, impl :128-200).
 * data, kernel: device pointers to p->dtype elements; out: device pointer
 * with room for the contiguous output (ndconv_output_shape). */
int ndconv_conv(const ndconv_problem *p, const void *data, const void *kernel, void *out,
                void *stream);

/* ConvFFTExt::conv_fft / conv_fft_with_processor / conv_fft_par
 * (src/conv_fft/mod.rs:81-183, impl :185-292, :394-423).
 * proc may be NULL (fresh-processor semantics); with a processor the
 * workspace, twiddle tables and a cached kernel spectrum are reused.
 * dtype F32, F64, C32, C64. */
int ndconv_conv_fft(const ndconv_problem *p, const void *data, const void *kernel, void *out,
                    ndconv_fft_processor *proc, void *stream);

/* Algorithm variants (autotuner candidates).  Every variant computes the same
 * convolution within the FFT path's tolerance (i32: direct only, exact).
 * No reference counterpart: the crate has one direct and one FFT method. */
typedef enum {
    NDCONV_ALGO_DIRECT = 0,           /* direct, FP32 FMA (sliding-window / tiled kernels) */
    NDCONV_ALGO_FFT = 1,              /* FFT, form and lengths picked by the cost model */
    NDCONV_ALGO_DIRECT_BF16X3 = 2,    /* direct, 3xBF16 split products on the tensor cores */
    NDCONV_ALGO_FFT_ND = 3,           /* FFT, full N-d transform, 7-smooth lengths */
    NDCONV_ALGO_FFT_RS = 4,           /* FFT along the contiguous axis, leading taps in the spectral domain */
    NDCONV_ALGO_FFT_ND_POW2 = 5,      /* as FFT_ND with power-of-two lengths */
    NDCONV_ALGO_FFT_RS_POW2 = 6,      /* as FFT_RS with power-of-two lengths */
    NDCONV_ALGO_COUNT = 7
} ndconv_algo;

/* One convolution by the given variant (ndconv_algo).  Direct variants
 * follow ConvExt::conv's argument rules, FFT variants ConvFFTExt::conv_fft's.
 * NDCONV_ERR_UNSUPPORTED when the variant does not apply (e.g. FFT of i32). */
int ndconv_conv_algo(const ndconv_problem *p, int32_t algo, const void *data, const void *kernel, void *out,
                     void *stream);

/* conv (algo 0) or conv_fft (algo 1) over n same-geometry instances whose
 * data, kernels and outputs are HOST arrays (contiguous): chunks of
 * instances are staged through library-owned device buffers so that
 * host->device copies, the convolution and device->host copies of
 * successive chunks overlap.  The overlap needs page-locked (pinned) host
 * arrays: with pageable ones each device->host copy blocks the calling
 * thread until its chunk's convolution has finished, so the chunks run one
 * after another (results are the same).  Asynchronous on `stream` for
 * pinned arrays: they must stay valid, and the outputs are complete, when
 * `stream` has synchronised.  A failing copy or launch returns its error.
 * No reference counterpart (the crate converts one host array per call). */
int ndconv_conv_batch_host(const ndconv_problem *p, int32_t algo, int64_t n, const void *const *data,
                           const void *const *kernel, void *const *out, ndconv_fft_processor *proc,
                           void *stream);

/* ConvExt::conv for f32 and Complex<f32> on the tensor cores (a complex
 * problem runs as four real convolutions of the interleaved parts, combined
 * as num-complex's product): 3xBF16 split products
 * (x k ~ xh kh + xh kl + xl kh) accumulated in f32, normwise error ~1e-6 vs
 * f64: row correlations of the padded data with groups of kernel rows on
 * the tensor cores, summed over each group's rows in the epilogue.  Any
 * strides, dilations, modes and borders (index ranges beyond the TMA
 * coordinate range: NDCONV_ERR_UNSUPPORTED); non-finite inputs fall back to
 * the FP32 loop so
 * NaN / Inf propagate as in the reference.  Same as
 * ndconv_conv_algo(p, NDCONV_ALGO_DIRECT_BF16X3, ...).  Asynchronous on
 * stream; a tensor-core pipeline wait that runs out (bounded at ~1 s, not
 * expected) leaves NaN in the affected output tile and is recorded in a
 * per-device word that ndconv_bf16x3_status reports. */
int ndconv_conv_bf16x3(const ndconv_problem *p, const void *data, const void *kernel, void *out, void *stream);
/* ndconv_conv_bf16x3 over n instances of one geometry (shapes, dilation,
 * modes) in one persistent launch: data / kernel / out are DEVICE arrays of n
 * device pointers (as ndconv_conv_batch).  The padded bf16 planes of all
 * instances are built first (stream-ordered workspace of ~4 bytes per
 * padded sample and instance), then every CTA takes tiles of any instance,
 * so small instances keep the tensor pipeline full.  Each instance's
 * result equals its ndconv_conv_bf16x3 call bit for bit.  A non-finite
 * value in any instance sends every instance through the FP32 loop.  No
 * reference counterpart (the crate convolves one array per call).  f32
 * only (NDCONV_ERR_UNSUPPORTED for other element types). */
int ndconv_conv_bf16x3_batch(const ndconv_problem *p, int64_t n, const void *const *data,
                             const void *const *kernel, void *const *out, void *stream);
/* Host only: the tile plan of ndconv_conv_bf16x3 for p (a complex
 * problem: its real views'), for tests and tuning.  out[0..15] = kernel
 * rows per group G, row groups, output columns per tile BN, MMA N = G BN,
 * K extent Kpad, 64-wide K chunks, 16-wide steps in the last chunk, output
 * rows per tile, ring stages, stage bytes, ring bytes (resident Toeplitz
 * tiles included), dynamic shared memory, Toeplitz tiles resident (0/1),
 * tiles along the middle axis, tiles along the contiguous axis, the shared
 * memory limit, then out[16..17] = outputs per virtual row S and virtual
 * rows R of a folded single row (0 and 1 when not folded: a single row --
 * a 1-D signal, or one row with one-row kernels -- is cut into R stretches
 * of S outputs that fill the tile's 128 accumulator lanes; the tile counts
 * before are those of the folded geometry).  No reference counterpart. */
int ndconv_bf16x3_plan(const ndconv_problem *p, int64_t out[18]);
/* Synchronises stream, then reports (NDCONV_ERR_TIMEOUT) and clears the
 * timeouts of every 3xBF16 launch on the current device since the last
 * call; NDCONV_OK when there were none.  No reference counterpart. */
int ndconv_bf16x3_status(void *stream);

/* Batched ConvExt::conv / ConvFFTExt::conv_fft over n instances that share
 * one problem geometry (shapes, dilation, modes); each instance has its
 * own data, kernel and output.  data / kernel / out are DEVICE arrays of n
 * device pointers.  The crate has no batch call: these are the loops
 * `for i in 0..n { x[i].conv(k[i], ..) }` and `.conv_fft(..)` in one
 * submission.  The FFT batch runs in waves whose spectra stay in L2. */
int ndconv_conv_batch(const ndconv_problem *p, int64_t n, const void *const *data,
                      const void *const *kernel, void *const *out, void *stream);
int ndconv_conv_fft_batch(const ndconv_problem *p, int64_t n, const void *const *data,
                          const void *const *kernel, void *const *out, ndconv_fft_processor *proc,
                          void *stream);

/* Heterogeneous batch: n independent problems (any shapes, kernels, modes,
 * element types), each run by the algorithm variant algo[i] (ndconv_algo:
 * 0 direct, 1 FFT, 2 direct on the tensor cores (3xBF16; other element
 * types run the FP32-family direct kernels), 3..6 the FFT plan variants).
 * No counterpart in the reference (its calls are one instance at a time).
 * data / kernel / out are HOST arrays of n device pointers, bound at
 * creation.  f32 instances become tasks of one persistent kernel driven by a
 * device-side work queue; others, and the tensor-core instances, run as
 * ordinary launches on a side stream in the same submission.  The plan owns
 * all spectra (allocated once); a tensor-core instance allocates its bf16
 * planes stream-ordered on each run. */
int ndconv_batch_create(const ndconv_problem *problems, int64_t n, const int32_t *algo,
                        const void *const *data, const void *const *kernel, void *const *out,
                        ndconv_batch_plan **plan);
/* Run the batch on stream; use_graph = 1 captures the submission into a
 * CUDA graph on first use and replays it afterwards. */
int ndconv_batch_run(ndconv_batch_plan *plan, int32_t use_graph, void *stream);
/* The same instances, one per-instance entry point call each (the plain
 * drop-in path), for comparison. */
int ndconv_batch_run_plain(ndconv_batch_plan *plan, void *stream);
/* Synchronises stream; NDCONV_ERR_TIMEOUT if a queue wait ran out (a task
 * whose predecessors did not finish within the poll bound gives up waiting,
 * runs, and the kernel returns normally). */
int ndconv_batch_status(ndconv_batch_plan *plan, void *stream);
/* Poll bound of the queue's dependency waits for later runs of the plan
 * (polls <= 0: the default, 2^24 polls, ~1-2 s).  No reference counterpart. */
int ndconv_batch_set_wait_limit(ndconv_batch_plan *plan, int64_t polls);
/* Test hook for the timeout path (no reference counterpart): enable = 1 makes
 * the plan's first waiting task wait on a counter that no task bumps, so
 * that its wait runs out after the poll bound and ndconv_batch_status
 * reports NDCONV_ERR_TIMEOUT; enable = 0 restores the task.  No GPU fault:
 * the task gives up, runs and the queue completes. */
int ndconv_batch_stall_one_wait(ndconv_batch_plan *plan, int32_t enable);
/* tasks, grid, shared bytes, #FFT, #direct, #standalone, workspace bytes, counters */
int ndconv_batch_info(const ndconv_batch_plan *plan, int64_t info[8]);
int ndconv_batch_destroy(ndconv_batch_plan *plan);

/* ndconv_conv_fft for callers that cannot allocate device memory (real-time
 * or embedded hosts that forbid allocation after start-up, plugins whose
 * host application owns every device allocation).  No counterpart in the
 * reference.  Same arguments and results as ndconv_conv_fft without a
 * processor, but the spectra and twiddle tables live in one fixed 16 MiB
 * device array that the library holds on every GPU where it is loaded; it
 * never calls cudaMalloc or cudaFree.  Problems whose spectra need more
 * than 16 MiB get NDCONV_ERR_NO_MEMORY.  One exception to "same results":
 * where no FFT form applies (a kernel row longer than the longest
 * overlap-save segment, leading axes too long for one column pass, rows of
 * 2^31 samples or more) ndconv_conv_fft runs the direct kernels, whose
 * axis-folding form allocates; this entry point returns
 * NDCONV_ERR_UNSUPPORTED there instead.  The first call on each device
 * looks up the array's address, so make it before any stream capture.
 * Calls share the array: calls whose GPU work overlaps race and must be
 * serialised by the caller. */
int ndconv_conv_fft_noalloc(const ndconv_problem *p, const void *data, const void *kernel, void *out,
                            void *stream);

/* GetProcessor::get_processor / get_fft_processor::<T, InElem>()
 * (src/conv_fft/processor/mod.rs:71-73,125-143; src/lib.rs:75-77).
 * dtype F32/F64 selects the real processor (real.rs), C32/C64 the complex
 * one (complex.rs). */
int ndconv_fft_processor_create(int32_t dtype, ndconv_fft_processor **out);
int ndconv_fft_processor_destroy(ndconv_fft_processor *proc);

/* Kernel-spectrum reuse (the crate sketches a "baked" processor in
 * commented-out code, src/conv_fft/mod.rs:22-42,306-392): transform `kernel`
 * (device pointer) for problem p once and keep its spectrum in proc; later
 * ndconv_conv_fft(p2, x, kernel, y, proc, s) calls whose geometry equals p's
 * (shapes, dilation, modes, padding; data strides may differ) and whose
 * kernel pointer equals `kernel` skip the kernel transform.  Bake again after
 * changing the kernel's contents. */
int ndconv_fft_processor_bake(ndconv_fft_processor *proc, const ndconv_problem *p, const void *kernel,
                              void *stream);

/* Processor::forward (src/conv_fft/processor/mod.rs:79-100; real.rs:24-155,
 * complex.rs:119-128).  Output layout is the reference's: axes rotated right
 * after each pass; out_shape receives it (query with out == NULL). */
int ndconv_fft_forward(ndconv_fft_processor *proc, int32_t rank, const int64_t shape[3],
                       const void *in, void *out, int64_t out_shape[3], void *stream);

/* Processor::backward (processor/mod.rs:102-119; real.rs:157-281,
 * complex.rs:131-144): inverse of forward, divided by the element count.
 * The real processor uses the last-axis length remembered by its last
 * forward call, like the reference's rp_origin_len. */
int ndconv_fft_backward(ndconv_fft_processor *proc, int32_t rank, const int64_t shape[3],
                        const void *in, void *out, int64_t out_shape[3], void *stream);

/* Number of CUDA kernels this library has launched in this process.
 * Diagnostics only; no counterpart in the reference. */
uint64_t ndconv_kernel_launches(void);

/* Planning facts for one problem (host only): out[0] modelled direct time
 * (s), out[1] modelled FFT time (s, 1e30 when the FFT passes do not fit a
 * persistent-kernel CTA), out[2] direct MACs, out[3] algorithmic bytes,
 * out[4..6] FFT lengths, out[7] 1 if the FFT fits.  No counterpart in the
 * reference; used by dispatchers. */
int ndconv_plan_info(const ndconv_problem *p, double out[8]);

/* Tile and plan parameters inside one algorithm, for the autotuner (no
 * reference counterpart).  Thread-local; value 0 (the default) lets the
 * library choose.  The FFT knobs never change results; the direct and
 * tensor-core ones may change the last bits (another summation chunking),
 * always within the same error bound.  Knob values that do not apply to a
 * problem are ignored for it.
 *   NDCONV_TUNE_SW_TY       warp row sets per CTA of the sliding-window
 *                           direct kernel (1, 2, 4, 8; at most 8 / dilation
 *                           phases)
 *   NDCONV_TUNE_MAC_ROWS    output rows per CTA of the FFT spectral tap sum
 *                           (1, 2, 4, 8)
 *   NDCONV_TUNE_ROW_THREADS threads of FFT row-pass CTAs in launches of many
 *                           CTAs (a multiple of 32, at most 512)
 *   NDCONV_TUNE_BF16X3_BN   output columns per tensor-core tile (16, 32 or
 *                           64; taken when it times the group's kernel rows
 *                           fits 256 MMA columns)
 *   NDCONV_TUNE_SW_RY       output rows per warp of the sliding-window
 *                           direct kernel (1, 2 or 4; f64 / c32 at most 2,
 *                           c64 1) */
typedef enum {
    NDCONV_TUNE_SW_TY = 0,
    NDCONV_TUNE_MAC_ROWS = 1,
    NDCONV_TUNE_ROW_THREADS = 2,
    NDCONV_TUNE_BF16X3_BN = 3,
    NDCONV_TUNE_SW_RY = 4,
    NDCONV_TUNE_COUNT = 5
} ndconv_tune_knob;
int ndconv_set_tuning(int32_t knob, int32_t value);
int32_t ndconv_get_tuning(int32_t knob);

/* Message for the last non-OK status returned on this thread. */
const char *ndconv_last_error(void);

/* Library version string. */
const char *ndconv_version(void);

/* ---- learned dispatcher network (no counterpart in the reference) -------
 * An MLP n_in -> n_hidden -> n_hidden -> n_out with ReLU, f32 parameters in
 * one flat device array (W1[h][in], b1[h], W2[h][h], b2[h], W3[out][h],
 * b3[out]).  Loss: sum over (sample, output) of mask * (y - target)^2 /
 * (2 * sum(mask)).  x, target, mask, y, grad: device pointers, row-major
 * [n][n_in] / [n][n_out]; loss: device pointer to one float (may be NULL). */
typedef struct ndconv_mlp ndconv_mlp;
int ndconv_mlp_create(int32_t n_in, int32_t n_hidden, int32_t n_out, uint64_t seed, ndconv_mlp **out);
int ndconv_mlp_destroy(ndconv_mlp *net);
int64_t ndconv_mlp_param_count(const ndconv_mlp *net);
/* copy all parameters to (set = 0) or from (set = 1) a host array of n floats */
int ndconv_mlp_params(ndconv_mlp *net, float *host, int64_t n, int32_t set);
int ndconv_mlp_forward(ndconv_mlp *net, const float *x, int64_t n, float *y, void *stream);
int ndconv_mlp_gradient(ndconv_mlp *net, const float *x, const float *target, const float *mask, int64_t n,
                        float *grad, float *loss, void *stream);
/* Adam over shuffled minibatches for `epochs` passes; final_loss (host
 * pointer, may be NULL) receives the loss over all n samples afterwards. */
int ndconv_mlp_train(ndconv_mlp *net, const float *x, const float *target, const float *mask, int64_t n,
                     int32_t epochs, int32_t batch, float lr, uint64_t seed, float *final_loss, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* NDCONV_H */
