// FFT convolution and processor entry points (host side).
#pragma once
#include "common.cuh"
#include "fft_core.cuh"

namespace ndconv {

// FFT plan variants (autotuner candidates): the form (full N-d transform,
// or row-spectral: FFT along the contiguous axis with the leading-axis taps
// summed in the spectral domain) and the transform lengths (7-smooth, or
// powers of two: radix-8/4/2 stages only).
enum FftVariant : int { FFTV_AUTO = 0, FFTV_ND = 1, FFTV_RS = 2, FFTV_ND_POW2 = 3, FFTV_RS_POW2 = 4 };

// conv_fft on the canonical geometry.  scratch (optional) must hold
// conv_fft_scratch_bytes(g) bytes; otherwise the processor's workspace or
// a stream-ordered allocation is used.
template <typename T>
int conv_fft_run(const Geom3<T> &g, int reverse, const T *x, const T *k, T *y,
                 ndconv_fft_processor *proc, cudaStream_t st, void *scratch, size_t scratch_bytes,
                 int variant = FFTV_AUTO);
template <typename T> size_t conv_fft_scratch_bytes(const Geom3<T> &g, int variant = FFTV_AUTO);
// Transform kernel k for geometry g into proc's baked spectrum; later
// conv_fft_run calls with proc, the same geometry and the same k pointer
// skip the kernel transform.
template <typename T>
int conv_fft_bake(const Geom3<T> &g, int reverse, const T *k, ndconv_fft_processor *proc, cudaStream_t st);
// n instances sharing the geometry; xs / ks / ys are device arrays of n
// device pointers.  Runs in waves whose spectra fit a share of L2.
template <typename T>
int conv_fft_batch_run(const Geom3<T> &g, int reverse, int64_t n, const T *const *xs, const T *const *ks,
                       T *const *ys, ndconv_fft_processor *proc, cudaStream_t st, int variant = FFTV_AUTO);

template <typename T>
int proc_forward(ndconv_fft_processor *proc, int rank, const int64_t *shape, const T *in,
                 typename CplxT<typename Elem<T>::Real>::type *out, cudaStream_t st);
template <typename T>
int proc_backward(ndconv_fft_processor *proc, int rank, const int64_t *spec_shape,
                  const typename CplxT<typename Elem<T>::Real>::type *in, T *out, int64_t *out_shape,
                  cudaStream_t st);

bool make_plan(int L, FftPlanDev &pl);
// relative cost of one Stockham stage per element, by radix
double stage_cost(int r);
// Twiddle table on the current device (cached per length, or carved from
// the calling thread's TwArena): kind 0: tw[t] = exp(-2 pi i t / L);
// kind 1: the stage table of *pl (make_plan(L)).
template <typename C> int get_twiddles(int L, const C **out, int kind = 0, const FftPlanDev *pl = nullptr);

// Optional home for twiddle tables: while a TwArenaScope is alive on the
// calling thread, tables are carved from `base` and generated on `st`
// instead of the process-wide cache (which allocates and synchronises).
struct TwArena {
    static constexpr int kMaxTables = 16;
    unsigned char *base;
    size_t cap, used;
    cudaStream_t st;
    int n;
    int len[kMaxTables], elem[kMaxTables], kind[kMaxTables];
    void *table[kMaxTables];
};
struct TwArenaScope {
    explicit TwArenaScope(TwArena *a);
    ~TwArenaScope();
    TwArena *prev;
};
int64_t smooth_size(int64_t n, bool even);
int64_t pow2_size(int64_t n, bool even);

}  // namespace ndconv

int64_t ndconv_proc_origin_len(const ndconv_fft_processor *p);
int32_t ndconv_proc_dtype(const ndconv_fft_processor *p);
