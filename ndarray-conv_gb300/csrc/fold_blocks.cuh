// Device-side pieces of the axis-folding form (see fold.cu): per-element
// bodies of the weight folding and the non-finite scan, and one GEMM tile.
// Shared by the ordinary launches (fold.cu) and the persistent batch queue.
#pragma once
#include <type_traits>

#include "common.cuh"
#include "direct.h"
#include "direct_blocks.cuh"
#include "fold.h"

namespace ndconv {
namespace foldk {

constexpr int FBM = 128, FBN = 64;
// K step of the GEMM (wider elements take shorter steps: two buffers of both
// operand tiles stay within the 48 KB of static shared memory)
template <typename T> constexpr int fbk() { return sizeof(T) > 8 ? 4 : (sizeof(T) > 4 ? 8 : 16); }
constexpr int FPM = FBM + 4, FPN = FBN + 4;  // padded rows: 16-byte aligned, fewer bank conflicts

// shared memory of one GEMM tile: two buffers of the A (FBK x FPM) and B
// (FBK x FPN) tiles
template <typename T> constexpr size_t gemm_smem() { return 2 * sizeof(T) * (size_t)fbk<T>() * (FPM + FPN); }

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

template <typename T> __host__ __device__ inline int64_t f1_count(const FoldParams &F) {
    return F.km * F.ax[F.f0].K * F.ax[F.f1].out * F.ax[F.f1].n;
}
template <typename T> __host__ __device__ inline int64_t f0_count(const FoldParams &F) { return F.cout * F.cin * F.km; }
__host__ __device__ inline int64_t scan_count(const FoldParams &F) {
    const AxisGeom *A = F.ax;
    return A[0].n * A[1].n * A[2].n + A[0].K * A[1].K * A[2].K;
}

// T1[tm][t0][of1][if1] = sum over t1 with map_f1(of1, t1) = if1 of kf[tm, t0, t1]
// (the taps of bucket (of1, if1) of the f1 table, ascending)
template <typename T>
__device__ __forceinline__ void f1_elem(const T *__restrict__ k, const FoldParams &F, T *__restrict__ T1, int64_t u) {
    using E = Elem<T>;
    const AxisGeom &A1 = F.ax[F.f1];
    const int64_t n1 = A1.n, o1n = A1.out, K0 = F.ax[F.f0].K;
    const int64_t i1 = u % n1, r = u / n1;
    const int64_t o1 = r % o1n, r2 = r / o1n;
    const int64_t t0 = r2 % K0, tm = r2 / K0;
    const int32_t *off = F.off[1] + o1 * (n1 + 1), *tap = F.tap[1] + o1 * A1.K;
    typename E::Acc acc = E::zero();
    for (int e = off[i1], e1 = off[i1 + 1]; e < e1; e++) E::add(acc, kf_at(k, F, tm, t0, (int64_t)tap[e]));
    T1[u] = E::out(acc);
}

// W[(of0, of1)][(if0, if1)][tm] = sum over t0 with map_f0(of0, t0) = if0 of T1[tm][t0][of1][if1]
template <typename T>
__device__ __forceinline__ void f0_elem(const T *__restrict__ T1, const FoldParams &F, T *__restrict__ W, int64_t u,
                                        bool l2) {
    using E = Elem<T>;
    const AxisGeom &A0 = F.ax[F.f0], &A1 = F.ax[F.f1];
    const int64_t n1 = A1.n, o1n = A1.out, K0 = A0.K;
    const int64_t tm = u % F.km, r = u / F.km;
    const int64_t ci = r % F.cin, co = r / F.cin;
    const int64_t i0 = ci / n1, i1 = ci % n1, o0 = co / o1n, o1 = co % o1n;
    const int32_t *off = F.off[0] + o0 * (A0.n + 1), *tap = F.tap[0] + o0 * K0;
    typename E::Acc acc = E::zero();
    for (int e = off[i0], e1 = off[i0 + 1]; e < e1; e++) {
        const T *p = T1 + ((tm * K0 + tap[e]) * o1n + o1) * n1 + i1;
        T v;
        if constexpr (std::is_same<T, float>::value) v = l2 ? __ldcg(p) : *p;
        else v = *p;  // only f32 runs inside the persistent queue
        E::add(acc, v);
    }
    W[u] = E::out(acc);
}

template <typename T> __device__ __forceinline__ bool finite_elem(T v) {
    if constexpr (Elem<T>::kInteger) return true;
    else if constexpr (Elem<T>::kComplex) return isfinite(v.re) && isfinite(v.im);
    else return isfinite(v);
}

// element u of the scan (data samples, then kernel taps): not finite?
template <typename T>
__device__ __forceinline__ bool scan_elem(const T *__restrict__ x, const T *__restrict__ k, const FoldParams &F,
                                          int64_t u) {
    const AxisGeom *A = F.ax;
    const int64_t nx = A[0].n * A[1].n * A[2].n;
    if (u < nx) {
        const int64_t i2 = u % A[2].n, r = u / A[2].n;
        const int64_t i1 = r % A[1].n, i0 = r / A[1].n;
        return !finite_elem(x[i0 * A[0].xs + i1 * A[1].xs + i2 * A[2].xs]);
    }
    const int64_t v = u - nx;
    const int64_t t2 = v % A[2].K, r = v / A[2].K;
    const int64_t t1 = r % A[1].K, t0 = r / A[1].K;
    return !finite_elem(k[t0 * A[0].ks + t1 * A[1].ks + t2 * A[2].ks]);
}

// Y[om][co] = sum over kk = (ci, tm) of X[om][kk] W[co][kk] for tile (bx, by):
// 128 x 64 outputs, 8 x 4 per thread (256 threads).  K advances in steps of
// FBK through two shared-memory buffers: the global loads of step s + 1 are
// in flight (in registers) while step s is multiplied, one barrier per step.
// A thread always loads the same K column kk = tid mod FBK of a step, so its
// tap position and data offset take one division per step.  The data operand
// is gathered through the border map.  Summation order: k ascending for every
// output, as in a plain loop.
// flag != 0 (a non-finite input): the reference's tap-by-tap sums instead.
template <typename T>
__device__ __forceinline__ void gemm_tile(const T *__restrict__ x, const T *__restrict__ W, T *__restrict__ y,
                                          const FoldParams &F, const int *flag, const T *__restrict__ k,
                                          const DirectParams<T> &fb, int64_t bx, int64_t by, unsigned char *smem,
                                          bool l2) {
    using E = Elem<T>;
    using Acc = typename E::Acc;
    constexpr int FBK = fbk<T>();
    constexpr int RA = FBM * FBK / 256, RB = FBN * FBK / 256;  // operand elements per thread and step
    constexpr int RS = 256 / FBK;                               // row step between a thread's elements
    T(*As)[FBK][FPM] = reinterpret_cast<T(*)[FBK][FPM]>(smem);
    T(*Bs)[FBK][FPN] = reinterpret_cast<T(*)[FBK][FPN]>(smem + 2 * sizeof(T) * FBK * FPM);
    const AxisGeom &Am = F.ax[F.m], &A0 = F.ax[F.f0], &A1 = F.ax[F.f1];
    const int64_t bm = bx * FBM, bn = by * FBN;
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    if (*reinterpret_cast<const volatile int *>(flag)) {
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
    const int kk = tid % FBK, r0 = tid / FBK;
    T ra[RA], rb[RB];
    // (channel, main-axis tap) of this thread's K column, advanced by FBK per
    // step without a division
    int ci = kk / km, tm = kk - (kk / km) * km;
    // this thread's operand elements of the step whose column is kg
    auto fetch = [&](int64_t kg) {
        const bool kin = kg < kdim;
        const int64_t kpos = (F.tlo_m + tm) * Am.d;
        const int64_t koff = (int64_t)(ci / n1) * A0.xs + (int64_t)(ci % n1) * A1.xs;
        // padded positions of the first and last row of the thread: all
        // inside the data (the usual case) -> plain strided loads
        const int64_t om0 = bm + r0, omL = bm + r0 + (RA - 1) * RS;
        const int64_t j0 = om0 * Am.s + kpos, jL = omL * Am.s + kpos;
        if (kin && j0 >= Am.p0 && jL < Am.p0 + Am.n && omL < Am.out) {
            const T *xp = x + (j0 - Am.p0) * Am.xs + koff;
            const int64_t step = (int64_t)RS * Am.s * Am.xs;
#pragma unroll
            for (int r = 0; r < RA; r++) ra[r] = xp[r * step];
        } else {
#pragma unroll
            for (int r = 0; r < RA; r++) {
                const int64_t om = om0 + r * RS;
                T v = E::zero();
                if (kin && om < Am.out) {
                    const int64_t mi = axis_map(Am, om * Am.s + kpos);
                    if (mi >= 0) v = x[mi * Am.xs + koff];
                }
                ra[r] = v;
            }
        }
#pragma unroll
        for (int r = 0; r < RB; r++) {
            const int64_t co = bn + r0 + r * RS;
            T w = E::zero();
            if (kin && co < F.cout) {
                const T *p = W + co * kdim + kg;
                if constexpr (std::is_same<T, float>::value) w = l2 ? __ldcg(p) : *p;
                else w = *p;  // only f32 runs inside the persistent queue
            }
            rb[r] = w;
        }
    };
    auto stash = [&](int buf) {
#pragma unroll
        for (int r = 0; r < RA; r++) As[buf][kk][r0 + r * RS] = ra[r];
#pragma unroll
        for (int r = 0; r < RB; r++) Bs[buf][kk][r0 + r * RS] = rb[r];
    };
    auto advance = [&]() {
        tm += FBK;
        while (tm >= km) {
            tm -= km;
            ci++;
        }
    };
    fetch(kk);
    stash(0);
    __syncthreads();
    int cur = 0;
    for (int64_t k0 = 0; k0 < kdim; k0 += FBK) {
        const bool more = k0 + FBK < kdim;
        if (more) {
            advance();
            fetch(k0 + FBK + kk);
        }
#pragma unroll
        for (int q = 0; q < FBK; q++) {
            T a[8], b[4];
            if constexpr (std::is_same<T, float>::value) {
                const float4 a0 = *reinterpret_cast<const float4 *>(&As[cur][q][ty * 8]);
                const float4 a1 = *reinterpret_cast<const float4 *>(&As[cur][q][ty * 8 + 4]);
                const float4 b0 = *reinterpret_cast<const float4 *>(&Bs[cur][q][tx * 4]);
                a[0] = a0.x, a[1] = a0.y, a[2] = a0.z, a[3] = a0.w;
                a[4] = a1.x, a[5] = a1.y, a[6] = a1.z, a[7] = a1.w;
                b[0] = b0.x, b[1] = b0.y, b[2] = b0.z, b[3] = b0.w;
            } else {
#pragma unroll
                for (int i = 0; i < 8; i++) a[i] = As[cur][q][ty * 8 + i];
#pragma unroll
                for (int j = 0; j < 4; j++) b[j] = Bs[cur][q][tx * 4 + j];
            }
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) E::mac(acc[i][j], a[i], b[j]);
        }
        if (more) stash(cur ^ 1);  // the other buffer: its readers finished before the last barrier
        __syncthreads();
        cur ^= 1;
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

}  // namespace foldk
}  // namespace ndconv
