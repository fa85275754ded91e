// Axis folding for direct convolution with all border constants zero.
//
// Along an axis with few input samples n and a long kernel (k_eff >> n) every
// tap reads one of only n samples (or a zero of the padding), so the taps of
// that axis can be summed per (output index, input index) before the
// convolution: with the other two canonical axes f0, f1 folded and m the
// remaining (main) axis,
//   y[om, of0, of1] = sum over (if0, if1) and main taps tm of
//                     W[(of0, of1)][(if0, if1)][tm] * x[map_m(om, tm), if0, if1]
//   W[(of0, of1)][(if0, if1)][tm] = sum of kf[tm, t0, t1] over the taps t0, t1
//                     with map_f0(of0, t0) = if0 and map_f1(of1, t1) = if1
// (kf the kernel in tap order, map the border map; taps reading padding
// zeros drop out).  That is a multi-channel 1-D convolution, computed as a
// GEMM (M = outputs along m, N = out_f0 out_f1, K = n_f0 n_f1 x main taps)
// with the data operand gathered through the border map.  Exact for i32
// (wrapping sums are order-free); for floats the summation order differs,
// and a non-finite input switches the GEMM to the plain per-output loop so
// NaN / Inf come out exactly as in the reference's tap-by-tap sums.
#include <cuda_runtime.h>

#include <type_traits>

#include "common.cuh"
#include "direct.h"
#include "direct_blocks.cuh"
#include "fold.h"
#include "fold_blocks.cuh"

namespace ndconv {

namespace {
using namespace foldk;

// tap tables of both folded axes: one thread per output index
__global__ void fold_tables_kernel(FoldParams F, int32_t *t0, int32_t *t1) {
    const AxisGeom &A0 = F.ax[F.f0], &A1 = F.ax[F.f1];
    const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u < A0.out) fold_table_row(A0, u, t0 + u * (A0.n + 1), t0 + A0.out * (A0.n + 1) + u * A0.K);
    else if (u < A0.out + A1.out) {
        const int64_t o = u - A0.out;
        fold_table_row(A1, o, t1 + o * (A1.n + 1), t1 + A1.out * (A1.n + 1) + o * A1.K);
    }
}

template <typename T>
__global__ void fold_f1_kernel(const T *__restrict__ k, FoldParams F, T *__restrict__ T1) {
    const int64_t total = f1_count<T>(F);
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x)
        f1_elem<T>(k, F, T1, u);
}

template <typename T>
__global__ void fold_f0_kernel(const T *__restrict__ T1, FoldParams F, T *__restrict__ W) {
    const int64_t total = f0_count<T>(F);
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x)
        f0_elem<T>(T1, F, W, u, false);
}

// flag |= 1 if any data sample or kernel tap is not finite
template <typename T>
__global__ void fold_scan_kernel(const T *__restrict__ x, const T *__restrict__ k, FoldParams F, int *flag) {
    const int64_t total = scan_count(F);
    bool bad = false;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x)
        bad |= scan_elem<T>(x, k, F, u);
    if (bad) atomicOr(flag, 1);
}

template <typename T>
__global__ void __launch_bounds__(256) fold_gemm_kernel(const T *__restrict__ x, const T *__restrict__ W,
                                                        T *__restrict__ y, FoldParams F, const int *flag,
                                                        const T *__restrict__ k, DirectParams<T> fb) {
    __shared__ __align__(16) unsigned char smem[gemm_smem<T>()];
    gemm_tile<T>(x, W, y, F, flag, k, fb, blockIdx.x, blockIdx.y, smem, false);
}
}  // namespace

template <typename T> bool plan_fold(const DirectParams<T> &P, FoldParams &F) {
    for (int a = 0; a < 3; a++)
        if (!host_zero(P.g.cf[a]) || !host_zero(P.g.cb[a])) return false;
    const AxisGeom *A = P.g.ax;
    double direct = 1;
    for (int a = 0; a < 3; a++) direct *= (double)A[a].out * (double)P.t_n[a];
    double best = -1;
    for (int m = 0; m < 3; m++) {
        const int f0 = m == 0 ? 1 : 0, f1 = m == 2 ? 1 : 2;
        if (A[f0].n > 256 || A[f1].n > 256 || P.t_n[m] < 1) continue;
        const double cin = (double)A[f0].n * A[f1].n, cout = (double)A[f0].out * A[f1].out, km = (double)P.t_n[m];
        if (cin > 4096 || cout * cin * km > (double)(1 << 26) || cout / FBN > 65535) continue;
        const double gemm = (double)A[m].out * cout * cin * km;
        const double prep = km * A[f0].K * A[f1].out * A[f1].n * A[f1].K + cout * cin * km * A[f0].K;
        const double c = gemm + 0.25 * prep;
        if (best < 0 || c < best) {
            best = c;
            F.m = m;
            F.f0 = f0;
            F.f1 = f1;
        }
    }
    if (best < 0 || best * 3 > direct) return false;
    for (int a = 0; a < 3; a++) F.ax[a] = A[a];
    F.reverse = P.reverse;
    F.tlo_m = P.t_lo[F.m];
    F.km = P.t_n[F.m];
    F.cin = A[F.f0].n * A[F.f1].n;
    F.cout = A[F.f0].out * A[F.f1].out;
    F.ys_m = P.ys_[F.m];
    F.ys_f0 = P.ys_[F.f0];
    F.ys_f1 = P.ys_[F.f1];
    return true;
}

template <typename T> size_t fold_scratch_bytes(const FoldParams &F) {
    const size_t w = (size_t)(F.cout * F.cin * F.km);
    const size_t t1 = (size_t)(F.km * F.ax[F.f0].K * F.ax[F.f1].out * F.ax[F.f1].n);
    const size_t tabs = (size_t)(fold_table_entries(F.ax[F.f0]) + fold_table_entries(F.ax[F.f1]));
    return sizeof(T) * (w + t1) + sizeof(int32_t) * tabs + 256;
}

void fold_set_tables(FoldParams &F, void *tables) {
    int32_t *t0 = static_cast<int32_t *>(tables);
    int32_t *t1 = t0 + fold_table_entries(F.ax[F.f0]);
    const AxisGeom &A0 = F.ax[F.f0], &A1 = F.ax[F.f1];
    F.off[0] = t0;
    F.tap[0] = t0 + A0.out * (A0.n + 1);
    F.off[1] = t1;
    F.tap[1] = t1 + A1.out * (A1.n + 1);
}

template <typename T>
cudaError_t fold_launch(const T *x, const T *k, T *y, const FoldParams &F, const DirectParams<T> &full,
                        cudaStream_t st, void *scratch, size_t scratch_bytes) {
    const size_t need = fold_scratch_bytes<T>(F);
    void *ws = scratch;
    if (!ws) {
        cudaError_t e = cudaMallocAsync(&ws, need, st);
        if (e != cudaSuccess) return e;
    } else if (scratch_bytes < need) {
        return cudaErrorInvalidValue;
    }
    T *W = static_cast<T *>(ws);
    T *T1 = W + F.cout * F.cin * F.km;
    int32_t *tabs = reinterpret_cast<int32_t *>(T1 + F.km * F.ax[F.f0].K * F.ax[F.f1].out * F.ax[F.f1].n);
    const int64_t ntab = fold_table_entries(F.ax[F.f0]) + fold_table_entries(F.ax[F.f1]);
    int *flag = reinterpret_cast<int *>((reinterpret_cast<uintptr_t>(tabs + ntab) + 15) & ~(uintptr_t)15);
    FoldParams Ft = F;
    fold_set_tables(Ft, tabs);
    cudaMemsetAsync(flag, 0, sizeof(int), st);
    {
        const int64_t rows = F.ax[F.f0].out + F.ax[F.f1].out;
        fold_tables_kernel<<<(unsigned)((rows + 127) / 128), 128, 0, st>>>(Ft, tabs,
                                                                          tabs + fold_table_entries(F.ax[F.f0]));
        ndconv_count_launch();
    }
    if (!Elem<T>::kInteger) {
        fold_scan_kernel<T><<<152 * 4, 256, 0, st>>>(x, k, F, flag);
        ndconv_count_launch();
    }
    fold_f1_kernel<T><<<152 * 8, 256, 0, st>>>(k, Ft, T1);
    fold_f0_kernel<T><<<152 * 8, 256, 0, st>>>(T1, Ft, W);
    dim3 grid((unsigned)((F.ax[F.m].out + FBM - 1) / FBM), (unsigned)((F.cout + FBN - 1) / FBN));
    fold_gemm_kernel<T><<<grid, 256, 0, st>>>(x, W, y, Ft, flag, k, full);
    ndconv_count_launch(3);
    cudaError_t e = cudaGetLastError();
    if (!scratch) cudaFreeAsync(ws, st);
    return e;
}

#define NDCONV_INST_FOLD(T)                                                                                \
    template bool plan_fold<T>(const DirectParams<T> &, FoldParams &);                                    \
    template size_t fold_scratch_bytes<T>(const FoldParams &);                                            \
    template cudaError_t fold_launch<T>(const T *, const T *, T *, const FoldParams &, const DirectParams<T> &, \
                                        cudaStream_t, void *, size_t);
NDCONV_INST_FOLD(float)
NDCONV_INST_FOLD(double)
NDCONV_INST_FOLD(int32_t)
NDCONV_INST_FOLD(int64_t)
NDCONV_INST_FOLD(c32)
NDCONV_INST_FOLD(c64)

}  // namespace ndconv
