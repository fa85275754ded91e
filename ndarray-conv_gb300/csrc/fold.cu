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

namespace ndconv {

namespace {
constexpr int FBM = 128, FBN = 64;

// border-mapped index of tap t for output o on an axis (-1: padding zero)
__device__ __forceinline__ int64_t fmap(const AxisGeom &A, int64_t o, int64_t t) {
    const int64_t i = axis_map(A, o * A.s + t * A.d);
    return i >= 0 ? i : -1;
}

template <typename T>
__device__ __forceinline__ T kf_at(const T *k, const FoldParams &F, int64_t tm, int64_t t0, int64_t t1) {
    int64_t t[3];
    t[F.m] = F.tlo_m + tm;
    t[F.f0] = t0;
    t[F.f1] = t1;
    int64_t off = 0;
    for (int a = 0; a < 3; a++) off += tap_source(t[a], F.ax[a].K, F.reverse) * F.ax[a].ks;
    return k[off];
}

// T1[tm][t0][of1][if1] = sum over t1 with map_f1(of1, t1) = if1 of kf[tm, t0, t1]
template <typename T>
__global__ void fold_f1_kernel(const T *__restrict__ k, FoldParams F, T *__restrict__ T1) {
    using E = Elem<T>;
    const AxisGeom &A1 = F.ax[F.f1];
    const int64_t n1 = A1.n, o1n = A1.out, K0 = F.ax[F.f0].K;
    const int64_t total = F.km * K0 * o1n * n1;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i1 = u % n1, r = u / n1;
        const int64_t o1 = r % o1n, r2 = r / o1n;
        const int64_t t0 = r2 % K0, tm = r2 / K0;
        typename E::Acc acc = E::zero();
        for (int64_t t1 = 0; t1 < A1.K; t1++)
            if (fmap(A1, o1, t1) == i1) E::add(acc, kf_at(k, F, tm, t0, t1));
        T1[u] = E::out(acc);
    }
}

// W[(of0, of1)][(if0, if1)][tm] = sum over t0 with map_f0(of0, t0) = if0 of T1[tm][t0][of1][if1]
template <typename T>
__global__ void fold_f0_kernel(const T *__restrict__ T1, FoldParams F, T *__restrict__ W) {
    using E = Elem<T>;
    const AxisGeom &A0 = F.ax[F.f0], &A1 = F.ax[F.f1];
    const int64_t n0 = A0.n, n1 = A1.n, o1n = A1.out, K0 = A0.K;
    const int64_t total = F.cout * F.cin * F.km;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t tm = u % F.km, r = u / F.km;
        const int64_t ci = r % F.cin, co = r / F.cin;
        const int64_t i0 = ci / n1, i1 = ci % n1, o0 = co / o1n, o1 = co % o1n;
        typename E::Acc acc = E::zero();
        for (int64_t t0 = 0; t0 < K0; t0++)
            if (fmap(A0, o0, t0) == i0) E::add(acc, T1[((tm * K0 + t0) * o1n + o1) * n1 + i1]);
        W[u] = E::out(acc);
    }
}

template <typename T> __device__ __forceinline__ bool finite_elem(T v) {
    if constexpr (std::is_same<T, int32_t>::value) return true;
    else if constexpr (Elem<T>::kComplex) return isfinite(v.re) && isfinite(v.im);
    else return isfinite(v);
}

// flag |= 1 if any data sample or kernel tap is not finite
template <typename T>
__global__ void fold_scan_kernel(const T *__restrict__ x, const T *__restrict__ k, FoldParams F, int *flag) {
    const AxisGeom *A = F.ax;
    const int64_t nx = A[0].n * A[1].n * A[2].n, nk = A[0].K * A[1].K * A[2].K;
    bool bad = false;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nx + nk; u += (int64_t)gridDim.x * blockDim.x) {
        if (u < nx) {
            const int64_t i2 = u % A[2].n, r = u / A[2].n;
            const int64_t i1 = r % A[1].n, i0 = r / A[1].n;
            bad |= !finite_elem(x[i0 * A[0].xs + i1 * A[1].xs + i2 * A[2].xs]);
        } else {
            const int64_t v = u - nx;
            const int64_t t2 = v % A[2].K, r = v / A[2].K;
            const int64_t t1 = r % A[1].K, t0 = r / A[1].K;
            bad |= !finite_elem(k[t0 * A[0].ks + t1 * A[1].ks + t2 * A[2].ks]);
        }
    }
    if (bad) atomicOr(flag, 1);
}

// Y[om][co] = sum over kk = (ci, tm) of X[om][kk] W[co][kk]: a 128 x 64
// tile per CTA, 8 x 4 outputs per thread, K in steps of 16 staged in shared
// memory.  The K slice's tap position and data offset (which depend on kk
// only) are tabulated once per step, so the data gather is one border map
// and one load per element.
template <typename T>
__global__ void __launch_bounds__(256) fold_gemm_kernel(const T *__restrict__ x, const T *__restrict__ W,
                                                        T *__restrict__ y, FoldParams F, const int *flag,
                                                        const T *__restrict__ k, DirectParams<T> fb) {
    using E = Elem<T>;
    using Acc = typename E::Acc;
    constexpr int FBK = sizeof(T) > 8 ? 8 : 16;  // keeps 16-byte types under 48 KB of static smem
    __shared__ T As[FBK][FBM + 1];
    __shared__ T Bs[FBK][FBN + 1];
    __shared__ int64_t kpos[FBK], koff[FBK];
    const AxisGeom &Am = F.ax[F.m], &A0 = F.ax[F.f0], &A1 = F.ax[F.f1];
    const int64_t bm = (int64_t)blockIdx.x * FBM, bn = (int64_t)blockIdx.y * FBN;
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    if (*reinterpret_cast<const volatile int *>(flag)) {
        // non-finite input: the reference's tap-by-tap sums for this tile
        for (int u = tid; u < FBM * FBN; u += 256) {
            const int64_t om = bm + u % FBM, co = bn + u / FBM;
            if (om >= Am.out || co >= F.cout) continue;
            int64_t o[3];
            o[F.m] = om;
            o[F.f0] = co / A1.out;
            o[F.f1] = co % A1.out;
            direct_naive_one<T>(x, k, y, fb, (o[0] * fb.g.ax[1].out + o[1]) * fb.g.ax[2].out + o[2]);
        }
        return;
    }
    Acc acc[8][4];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = E::zero();
    const int64_t kdim = F.cin * F.km;
    const int km = (int)F.km, n1 = (int)A1.n;
    for (int64_t k0 = 0; k0 < kdim; k0 += FBK) {
        if (tid < FBK) {
            const int64_t kg = k0 + tid;
            const int ci = (int)(kg / km), tm = (int)(kg - (int64_t)ci * km);
            kpos[tid] = (F.tlo_m + tm) * Am.d;
            koff[tid] = (kg < kdim) ? (int64_t)(ci / n1) * A0.xs + (int64_t)(ci % n1) * A1.xs : -1;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < FBM * FBK / 256; r++) {
            const int idx = tid + r * 256;
            const int kk = idx % FBK, row = idx / FBK;
            const int64_t om = bm + row;
            T v = E::zero();
            if (koff[kk] >= 0 && om < Am.out) {
                const int64_t mi = axis_map(Am, om * Am.s + kpos[kk]);
                if (mi >= 0) v = x[mi * Am.xs + koff[kk]];
            }
            As[kk][row] = v;
        }
#pragma unroll
        for (int r = 0; r < FBN * FBK / 256; r++) {
            const int idx = tid + r * 256;
            const int kk = idx % FBK, col = idx / FBK;
            const int64_t kg = k0 + kk, co = bn + col;
            Bs[kk][col] = (kg < kdim && co < F.cout) ? W[co * kdim + kg] : E::zero();
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < FBK; kk++) {
            T a[8], b[4];
#pragma unroll
            for (int i = 0; i < 8; i++) a[i] = As[kk][ty * 8 + i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) E::mac(acc[i][j], a[i], b[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int64_t om = bm + ty * 8 + i;
        if (om >= Am.out) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int64_t co = bn + tx * 4 + j;
            if (co >= F.cout) continue;
            y[om * F.ys_m + (co / A1.out) * F.ys_f0 + (co % A1.out) * F.ys_f1] = E::out(acc[i][j]);
        }
    }
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
        if (A[f0].n > 256 || A[f1].n > 256) continue;
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
    return sizeof(T) * (w + t1) + 256;
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
    int *flag = reinterpret_cast<int *>((reinterpret_cast<uintptr_t>(T1 + F.km * F.ax[F.f0].K * F.ax[F.f1].out *
                                                                          F.ax[F.f1].n) + 15) & ~(uintptr_t)15);
    cudaMemsetAsync(flag, 0, sizeof(int), st);
    if (!std::is_same<T, int32_t>::value) {
        fold_scan_kernel<T><<<152 * 4, 256, 0, st>>>(x, k, F, flag);
        ndconv_count_launch();
    }
    fold_f1_kernel<T><<<152 * 8, 256, 0, st>>>(k, F, T1);
    fold_f0_kernel<T><<<152 * 8, 256, 0, st>>>(T1, F, W);
    dim3 grid((unsigned)((F.ax[F.m].out + FBM - 1) / FBM), (unsigned)((F.cout + FBN - 1) / FBN));
    fold_gemm_kernel<T><<<grid, 256, 0, st>>>(x, W, y, F, flag, k, full);
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
NDCONV_INST_FOLD(c32)
NDCONV_INST_FOLD(c64)

}  // namespace ndconv
