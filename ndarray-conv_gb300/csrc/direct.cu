// Direct N-d convolution (ConvExt::conv, src/conv/mod.rs:128-200) on sm_103a.
//
// One CTA computes a TY x TX tile of one output plane.  The padded input
// is never materialised: for every chunk of kernel taps the CTA stages the
// window of the padded input it needs in shared memory, evaluating each
// padded position with the closed-form border map (axis_map) straight from
// the unpadded data, then every thread accumulates RX outputs of one row
// (columns tx, tx+BX, ...) over the chunk's taps.  Taps follow the
// reference's order (row-major over the reversed kernel, dilation as the
// tap stride), and exact-zero taps are skipped like gen_offset_list
// (src/dilation/mod.rs:47-50); the skip is warp-uniform.
#include "common.cuh"
#include "direct.h"
#include "direct_blocks.cuh"
#include "fold.h"

#include <type_traits>

namespace ndconv {

// CTA (bx, by, bz) of the tiled kernel; block shape (BX, BY) comes from P.
template <typename T>
__global__ void __launch_bounds__(256) dead_tap_fixup_kernel(const T *__restrict__ k0, T *__restrict__ y0,
                                                             const __grid_constant__ DirectParams<T> P) {
    const int64_t inst = blockIdx.y;
    const T *k = P.ks ? P.ks[P.inst_base + inst] : k0;
    T *y = P.ys ? P.ys[P.inst_base + inst] : y0;
    dead_tap_fixup_block<T>(k, y, P, blockIdx.x, gridDim.x);
}

namespace {
bool sw_disabled() {
    static int v = -1;
    if (v < 0) {
        const char *e = getenv("NDCONV_DIRECT_NO_SW");
        v = (e && atoi(e)) ? 1 : 0;
    }
    return v == 1;
}

template <typename T>
cudaError_t launch_main(const T *x, const T *k, T *y, DirectParams<T> &P, cudaStream_t st, int force_naive,
                        int64_t n_inst) {
    const AxisGeom &A0 = P.g.ax[0], &A1 = P.g.ax[1], &A2 = P.g.ax[2];
    int BX = 0, BY = 0;
    const bool grid_ok = A0.out * n_inst < 65536 && (A1.out + 7) / 8 < 65536;
    if (!force_naive && grid_ok && A1.out < 65536 && !sw_disabled()) {
        // unit x-stride: sliding register windows
        constexpr int SRX = (sizeof(T) <= 4) ? 8 : 4;
        if (plan_sw(P, SRX, n_inst)) return launch_sw<T, SRX, 2 * SRX>(x, k, y, P, st, n_inst);
    }
    if (!force_naive && grid_ok) {
        if (plan_tile(P, 4, BX, BY)) return launch_tile<T, 4>(x, k, y, P, BX, BY, st, n_inst);
        if (plan_tile(P, 1, BX, BY)) return launch_tile<T, 1>(x, k, y, P, BX, BY, st, n_inst);
    }
    const int64_t total = A0.out * A1.out * A2.out;
    int64_t blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (n_inst > 65535) return cudaErrorInvalidConfiguration;
    direct_naive_kernel<T><<<dim3((unsigned)blocks, (unsigned)n_inst), 256, 0, st>>>(x, k, y, P);
    ndconv_count_launch();
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_any(const T *x, const T *k, T *y, DirectParams<T> P, cudaStream_t st, int force_naive,
                       int64_t n_inst, void *scratch = nullptr, size_t scratch_bytes = 0) {
    const AxisGeom &A0 = P.g.ax[0], &A1 = P.g.ax[1], &A2 = P.g.ax[2];
    if (A0.out <= 0 || A1.out <= 0 || A2.out <= 0 || n_inst <= 0) return cudaSuccess;
    if (!force_naive) {
        const DirectParams<T> full = P;
        restrict_live_taps(P);
        FoldParams F;
        if (n_inst == 1 && !P.xs && plan_fold(P, F))
            return fold_launch<T>(x, k, y, F, full, st, scratch, scratch_bytes);
        permute_axes_for_tiles(P);
    }
    cudaError_t e = launch_main<T>(x, k, y, P, st, force_naive, n_inst);
    if (e != cudaSuccess || !taps_restricted(P) || Elem<T>::kInteger) return e;
    // skipped taps with a non-finite weight: every output is NaN, as in the reference
    const int64_t nk = A0.K * A1.K;  // kernel rows
    int64_t parts = (nk + 255) / 256;
    if (parts > 64) parts = 64;
    dead_tap_fixup_kernel<T><<<dim3((unsigned)parts, (unsigned)n_inst), 256, 0, st>>>(k, y, P);
    ndconv_count_launch();
    return cudaGetLastError();
}
}  // namespace

template <typename T>
cudaError_t direct_conv_launch(const T *x, const T *k, T *y, DirectParams<T> P, cudaStream_t st,
                               int force_naive, void *scratch, size_t scratch_bytes) {
    P.xs = nullptr;
    P.ks = nullptr;
    P.ys = nullptr;
    P.inst_base = 0;
    return launch_any<T>(x, k, y, P, st, force_naive, 1, scratch, scratch_bytes);
}

template <typename T> size_t direct_scratch_bytes(DirectParams<T> P) {
    restrict_live_taps(P);
    FoldParams F;
    return plan_fold(P, F) ? fold_scratch_bytes<T>(F) : 0;
}

template <typename T>
cudaError_t direct_conv_batch_launch(int64_t n, const T *const *xs, const T *const *ks, T *const *ys,
                                     DirectParams<T> P, cudaStream_t st) {
    P.xs = xs;
    P.ks = ks;
    P.ys = ys;
    // chunks whose (instance, plane) count fits grid.z
    const int64_t per = (P.g.ax[0].out > 0) ? (65535 / P.g.ax[0].out) : 1;
    const int64_t chunk = per < 1 ? 1 : per;
    for (int64_t b = 0; b < n; b += chunk) {
        P.inst_base = b;
        const int64_t cnt = (n - b < chunk) ? n - b : chunk;
        cudaError_t e = launch_any<T>(nullptr, nullptr, nullptr, P, st, 0, cnt);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

#define NDCONV_INST_DIRECT_BATCH(T) \
    template cudaError_t direct_conv_batch_launch<T>(int64_t, const T *const *, const T *const *, T *const *, \
                                                     DirectParams<T>, cudaStream_t);
NDCONV_INST_DIRECT_BATCH(float)
NDCONV_INST_DIRECT_BATCH(double)
NDCONV_INST_DIRECT_BATCH(int32_t)
NDCONV_INST_DIRECT_BATCH(int64_t)
NDCONV_INST_DIRECT_BATCH(c32)
NDCONV_INST_DIRECT_BATCH(c64)
#define NDCONV_INST_DIRECT(T)                                                                             \
    template cudaError_t direct_conv_launch<T>(const T *, const T *, T *, DirectParams<T>, cudaStream_t, int, \
                                               void *, size_t);                                            \
    template size_t direct_scratch_bytes<T>(DirectParams<T>);
NDCONV_INST_DIRECT(float)
NDCONV_INST_DIRECT(double)
NDCONV_INST_DIRECT(int32_t)
NDCONV_INST_DIRECT(int64_t)
NDCONV_INST_DIRECT(c32)
NDCONV_INST_DIRECT(c64)

}  // namespace ndconv
