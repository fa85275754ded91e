// Direct-convolution CTA bodies and their tile planners, shared by the
// standalone kernels (direct.cu) and the persistent batch kernel.
#pragma once
#include <cstring>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "direct.h"

namespace ndconv {

template <typename T, int RX>
__device__ __forceinline__ void direct_tile_block(const T *__restrict__ x0, const T *__restrict__ k0,
                                                  T *__restrict__ y0, const DirectParams<T> &P, unsigned bx,
                                                  unsigned by, unsigned bz, unsigned char *smem_raw) {
    using E = Elem<T>;
    using Acc = typename E::Acc;
    // bz enumerates (instance, output plane)
    const int64_t inst = bz / P.g.ax[0].out;
    const T *__restrict__ x = P.xs ? P.xs[P.inst_base + inst] : (P.x1 ? P.x1 : x0);
    const T *__restrict__ k = P.ks ? P.ks[P.inst_base + inst] : (P.k1 ? P.k1 : k0);
    T *__restrict__ y = P.ys ? P.ys[P.inst_base + inst] : (P.y1 ? P.y1 : y0);
    const Geom3<T> &g = P.g;
    const AxisGeom &A0 = g.ax[0], &A1 = g.ax[1], &A2 = g.ax[2];
    const int BX = P.tile_bx, BY = P.tile_by;
    const int tx = threadIdx.x % BX, ty = threadIdx.x / BX;
    const int tid = ty * BX + tx, nthr = BX * BY;
    const int TX = BX * RX;

    T *tile = reinterpret_cast<T *>(smem_raw);
    T *wsm = tile + P.tile_elems;
    int64_t *mrow = reinterpret_cast<int64_t *>(smem_raw + P.maps_off);
    int64_t *mcol = mrow + P.max_rows;

    const int64_t oz = bz - inst * A0.out;
    const int64_t oy0 = (int64_t)by * BY;
    const int64_t ox0 = (int64_t)bx * TX;

    Acc acc[RX];
#pragma unroll
    for (int r = 0; r < RX; r++) acc[r] = E::zero();

    const int64_t s1 = A1.s, s2 = A2.s, d1 = A1.d, d2 = A2.d;
    // live taps only (taps outside [t_lo, t_lo + t_n) read padding zeros for every output)
    const int64_t kz_end = P.t_lo[0] + P.t_n[0], ky_end = P.t_lo[1] + P.t_n[1], kx_end = P.t_lo[2] + P.t_n[2];
    for (int64_t kz = P.t_lo[0]; kz < kz_end; kz++) {
        const int64_t mz = axis_map(A0, oz * A0.s + kz * A0.d);
        const int64_t kzs = tap_source(kz, A0.K, P.reverse);
        for (int64_t ky0 = P.t_lo[1]; ky0 < ky_end; ky0 += P.cky) {
            const int cky = (int)(P.cky < ky_end - ky0 ? P.cky : ky_end - ky0);
            const int64_t row0 = oy0 * s1 + ky0 * d1;
            const int nrows = (int)((BY - 1) * s1 + (cky - 1) * d1 + 1);
            for (int64_t kx0 = P.t_lo[2]; kx0 < kx_end; kx0 += P.ckx) {
                const int ckx = (int)(P.ckx < kx_end - kx0 ? P.ckx : kx_end - kx0);
                const int64_t col0 = ox0 * s2 + kx0 * d2;
                const int ncols = (int)((TX - 1) * s2 + (ckx - 1) * d2 + 1);
                __syncthreads();  // previous chunk's compute is done with smem
                for (int i = tid; i < nrows; i += nthr) mrow[i] = axis_map(A1, row0 + i);
                for (int i = tid; i < ncols; i += nthr) mcol[i] = axis_map(A2, col0 + i);
                for (int i = tid; i < cky * ckx; i += nthr) {
                    const int a = i / ckx, b = i - a * ckx;
                    const int64_t ys = tap_source(ky0 + a, A1.K, P.reverse);
                    const int64_t xs_ = tap_source(kx0 + b, A2.K, P.reverse);
                    wsm[i] = k[kzs * A0.ks + ys * A1.ks + xs_ * A2.ks];
                }
                __syncthreads();
                const int W = ncols;
                for (int i = tid; i < nrows * ncols; i += nthr) {
                    const int r = i / ncols, c = i - r * ncols;
                    tile[r * W + c] = resolve_padded<T>(x, g, mz, mrow[r], mcol[c]);
                }
                __syncthreads();
                const int is1 = (int)s1, id1 = (int)d1, is2 = (int)s2, id2 = (int)d2;
                for (int a = 0; a < cky; a++) {
                    const T *trow = tile + (ty * is1 + a * id1) * W + tx * is2;
                    for (int b = 0; b < ckx; b++) {
                        const T w = wsm[a * ckx + b];
                        if (E::is_zero(w)) continue;
                        const T *tp = trow + b * id2;
#pragma unroll
                        for (int r = 0; r < RX; r++) E::mac(acc[r], tp[r * BX * is2], w);
                    }
                }
            }
        }
    }
    const int64_t oy = oy0 + ty;
    if (oy < A1.out) {
        T *yrow = y + oz * P.ys_[0] + oy * P.ys_[1];
#pragma unroll
        for (int r = 0; r < RX; r++) {
            const int64_t ox = ox0 + tx + (int64_t)r * BX;
            if (ox < A2.out) yrow[ox * P.ys_[2]] = E::out(acc[r]);
        }
    }
}

template <typename T, int RX>
__global__ void __launch_bounds__(256) direct_tile_kernel(const T *__restrict__ x0, const T *__restrict__ k0,
                                                          T *__restrict__ y0, const __grid_constant__ DirectParams<T> P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    direct_tile_block<T, RX>(x0, k0, y0, P, blockIdx.x, blockIdx.y, blockIdx.z, smem_raw);
}

// CKX consecutive tap weights from shared memory as 16-byte vectors (the
// weight slots are 16-byte aligned and padded to whole chunks).
template <typename T, int N> __device__ __forceinline__ void load_taps(T (&w)[N], const T *p) {
    static_assert(sizeof(T) <= 16 && 16 % sizeof(T) == 0, "tap vectors hold whole elements");
    constexpr int PER = 16 / sizeof(T);
    static_assert(N % PER == 0, "tap chunks are whole vectors");
#pragma unroll
    for (int v = 0; v < N / PER; v++) {
        const uint4 u = reinterpret_cast<const uint4 *>(p)[v];
        memcpy(&w[v * PER], &u, 16);
    }
}

// One element global -> shared without passing through registers
// (cp.async, completed by cp.async.wait_all); 4-byte pieces, so only the
// element types' natural 4-byte alignment is assumed.
template <typename T> __device__ __forceinline__ void stage_async(T *smem, const T *gmem) {
    static_assert(sizeof(T) % 4 == 0, "elements of whole 4-byte words");
#pragma unroll
    for (int b = 0; b < (int)sizeof(T); b += 4) {
        const unsigned sa = (unsigned)__cvta_generic_to_shared(reinterpret_cast<char *>(smem) + b);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa),
                     "l"(reinterpret_cast<const char *>(gmem) + b)
                     : "memory");
    }
}

// acc[r] += win[r + t] w[t] over taps t of [O, O + B), r < RX.
template <typename E, int RX, int O, int B, typename Acc, typename T, int NW, int NT>
__device__ __forceinline__ void fma_taps(Acc (&acc)[RX], const T (&win)[NW], const T (&w)[NT]) {
#pragma unroll
    for (int t = O; t < O + B; t++)
#pragma unroll
        for (int r = 0; r < RX; r++) E::mac(acc[r], win[r + t], w[t]);
}

// The first m taps (0 < m < 2B) of a chunk whose first O are done, without a
// branch per tap: the binary digits of m from B down, each a compile-time
// block of taps, in ascending tap order.
template <typename E, int RX, int B, int O, typename Acc, typename T, int NW, int NT>
__device__ __forceinline__ void fma_tail(Acc (&acc)[RX], const T (&win)[NW], const T (&w)[NT], int m) {
    if constexpr (B >= 1) {
        if (m & B) {
            fma_taps<E, RX, O, B>(acc, win, w);
            fma_tail<E, RX, B / 2, O + B>(acc, win, w, m);
        } else {
            fma_tail<E, RX, B / 2, O>(acc, win, w, m);
        }
    }
}

// Sliding-window variant along the contiguous axis, any stride s and
// dilation d (g = gcd(s, d), D = d / g phases, S = s / g tap residues).
// Output ox = X0 + phi + D j, tap u = rho + S t of a chunk starting at kx0
// reads padded column X0 s + kx0 d + rho d + s (phi + D (j + t)), so for
// every (residue rho, phase phi) the outputs are an undilated unit-stride
// 1-D correlation over the decimated sequence
//   G[rho][phi][m] = row[X0 s + kx0 d + rho d + s (phi + D m)]
// with the taps rho, rho + S, ...  (s = 1: one residue, D = d phases).  A
// warp owns one (row set, phase, segment) line: RY output rows
// oy0 + ty + i TY (i < RY), 32 * RX outputs of each; lane l owns RX
// consecutive phase outputs j = l*RX + r of every row and slides a register
// window over G, so each shared-memory load feeds up to CKX FMAs per row.
// When TY s1 = H d1 the rows' input rows coincide: row i under kernel row a
// reads staged row ty s1 + (i H + a) d1, so one window serves every (i, a)
// with i H + a = j, and each staged row feeds up to RY kernel rows.  G is
// stored swizzled (element m at (m % RX) * Q + m / RX) so the lanes' window
// loads hit consecutive banks.  Every output accumulates its taps in the
// same order whatever TY and RY are: kz, then ky, then (residue, kx).
template <typename T, int RX, int CKX, int RYM>
__device__ __forceinline__ void direct_sw_block(const T *__restrict__ x0, const T *__restrict__ k0,
                                                T *__restrict__ y0, const DirectParams<T> &P, unsigned bx,
                                                unsigned by, unsigned bz, unsigned char *smem_raw) {
    using E = Elem<T>;
    using Acc = typename E::Acc;
    const AxisGeom &A0 = P.g.ax[0], &A1 = P.g.ax[1], &A2 = P.g.ax[2];
    const int64_t inst = bz / A0.out;
    const T *__restrict__ x = P.xs ? P.xs[P.inst_base + inst] : (P.x1 ? P.x1 : x0);
    const T *__restrict__ k = P.ks ? P.ks[P.inst_base + inst] : (P.k1 ? P.k1 : k0);
    T *__restrict__ y = P.ys ? P.ys[P.inst_base + inst] : (P.y1 ? P.y1 : y0);
    const int D = P.sw_ph;              // phases
    const int S = P.sw_res;             // tap residues
    const int TR = P.sw_tr;             // weight slots per residue (whole CKX chunks)
    const int SD = S * D;
    const int TY = P.sw_ty, NSEG = P.sw_nseg;
    const int RY = P.sw_ry, H = P.sw_h;  // rows per line, staged-row step between them
    const int SEGW = 32 * RX;           // phase outputs per line
    const int Q = P.sw_q;               // swizzle pitch
    const int PH = RX * Q;              // smem elements per (residue, phase) of one row
    const int ROWE = SD * PH;           // smem elements per staged row
    T *tile = reinterpret_cast<T *>(smem_raw);
    T *wsm = tile + P.tile_elems;
    int64_t *mrow = reinterpret_cast<int64_t *>(smem_raw + P.maps_off);
    int64_t *mcol = mrow + P.max_rows;
    int64_t *rowoff = mcol + P.max_cols;
    int *zrow = reinterpret_cast<int *>(rowoff + P.max_rows);
    int *dcol = zrow + P.cky;  // per staged column: its slot in a staged row
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nlines = TY * NSEG * D;
    const int ty = warp / (NSEG * D);
    const int sg = (warp / D) % NSEG;
    const int phi = warp % D;
    const int64_t oz = bz - inst * A0.out;
    const int64_t oy0 = (int64_t)by * TY * RY;
    const int64_t TXo = (int64_t)NSEG * D * SEGW;
    const int64_t X0 = (int64_t)bx * TXo;
    const int s1 = (int)A1.s, d1 = (int)A1.d;
    const int64_t s2 = A2.s, d2 = A2.d;

    Acc acc[RYM][RX];
#pragma unroll
    for (int i = 0; i < RYM; i++)
#pragma unroll
        for (int r = 0; r < RX; r++) acc[i][r] = E::zero();

    // live taps only (taps outside [t_lo, t_lo + t_n) read padding zeros for every output)
    const int64_t kz_end = P.t_lo[0] + P.t_n[0], ky_end = P.t_lo[1] + P.t_n[1], kx_end = P.t_lo[2] + P.t_n[2];
    for (int64_t kz = P.t_lo[0]; kz < kz_end; kz++) {
        const int64_t mz = axis_map(A0, oz * A0.s + kz * A0.d);
        const int64_t kzs = tap_source(kz, A0.K, P.reverse);
        for (int64_t ky0 = P.t_lo[1]; ky0 < ky_end; ky0 += P.cky) {
            const int cky = (int)(P.cky < ky_end - ky0 ? P.cky : ky_end - ky0);
            const int64_t row0 = oy0 * s1 + ky0 * d1;
            const int nrows = (TY * RY - 1) * s1 + (cky - 1) * d1 + 1;
            for (int64_t kx0 = P.t_lo[2]; kx0 < kx_end; kx0 += P.ckx) {
                const int ckx = (int)(P.ckx < kx_end - kx0 ? P.ckx : kx_end - kx0);
                const int tr0 = (ckx + S - 1) / S;          // taps of residue 0 (the most)
                const int64_t col0 = X0 * s2 + kx0 * d2;
                const int mlen = NSEG * SEGW + tr0 - 1;     // decimated elements per (residue, phase)
                const int ncols = SD * mlen;
                __syncthreads();
                // per staged row: data offset of an interior row, or -1 (then the
                // general border resolution is used); per column: mapped index
                for (int i = tid; i < nrows; i += blockDim.x) {
                    const int64_t my = axis_map(A1, row0 + i);
                    mrow[i] = my;
                    rowoff[i] = (mz >= 0 && my >= 0) ? mz * A0.xs + my * A1.xs : -1;
                }
                // column cc = (m, rho, phi) with (rho, phi) fastest: neighbouring
                // threads read neighbouring columns
                for (int i = tid; i < ncols; i += blockDim.x) {
                    const int m = (SD == 1) ? i : i / SD;
                    const int rem = i - m * SD;
                    const int rho = rem / D, ph = rem - rho * D;
                    mcol[i] = axis_map(A2, col0 + rho * d2 + s2 * (ph + (int64_t)D * m));
                    // swizzled slot (rho * D + phi) * PH + (m mod RX) * Q + m / RX, worked
                    // out once per column instead of once per staged element
                    dcol[i] = rem * PH + (m & (RX - 1)) * Q + m / RX;
                }
                for (int i = tid; i < cky; i += blockDim.x) zrow[i] = 0;
                __syncthreads();
                for (int i = tid; i < cky * S * TR; i += blockDim.x) {
                    const int a = i / (S * TR), rem = i - a * (S * TR);
                    const int rho = rem / TR, t = rem - rho * TR;
                    const int u = rho + S * t;
                    T w = E::zero();
                    if (u < ckx) {
                        w = k[kzs * A0.ks + tap_source(ky0 + a, A1.K, P.reverse) * A1.ks +
                              tap_source(kx0 + u, A2.K, P.reverse) * A2.ks];
                        if (E::is_zero(w)) zrow[a] = 1;  // this kernel row has taps to skip
                    }
                    wsm[i] = w;
                }
                __syncthreads();
                // every interior sample is copied asynchronously (all of a
                // thread's copies in flight at once); border samples are
                // resolved and stored
                const int64_t xs2 = A2.xs;
                for (int cc = tid; cc < ncols; cc += blockDim.x) {
                    const int64_t mc = mcol[cc];
                    T *dst = tile + dcol[cc];
                    const T *src = x + mc * xs2;
                    for (int rr = 0; rr < nrows; rr++) {
                        const int64_t ro = rowoff[rr];
                        if (ro >= 0 && mc >= 0) stage_async(dst + rr * ROWE, src + ro);
                        else dst[rr * ROWE] = resolve_padded<T>(x, P.g, mz, mrow[rr], mc);
                    }
                }
                asm volatile("cp.async.wait_all;\n" ::: "memory");
                __syncthreads();
                if (warp < nlines) {
                    // lane's first decimated element is a multiple of RX, and so is
                    // every chunk start t0, so element jbase + t0 + q sits at
                    // (q % RX) * Q + (jbase + t0) / RX + q / RX
                    const int lbase = sg * (SEGW / RX) + lane;
                    const int nj = (RY - 1) * H + cky;  // staged rows this line reads
                    for (int j = 0; j < nj; j++) {
                        const T *prow_j = tile + (ty * s1 + j * d1) * ROWE + phi * PH + lbase;
                        for (int rho = 0; rho < S; rho++) {
                            const T *prow = prow_j + rho * D * PH;
                            const int ckr = (ckx - rho + S - 1) / S;  // taps of this residue
                            for (int t0 = 0; t0 < ckr; t0 += CKX) {
                                T win[RX + CKX - 1];
                                const T *pw = prow + t0 / RX;
                                const bool full = t0 + CKX <= ckr;
                                if (full) {
                                    // every window element exists: one base pointer per
                                    // window residue, the rest immediate offsets
                                    const T *pr[RX];
#pragma unroll
                                    for (int r = 0; r < RX; r++) pr[r] = pw + r * Q;
#pragma unroll
                                    for (int q = 0; q < RX + CKX - 1; q++) win[q] = pr[q % RX][q / RX];
                                } else {
#pragma unroll
                                    for (int q = 0; q < RX + CKX - 1; q++)
                                        win[q] = (t0 + q < ckr + RX - 1) ? pw[(q % RX) * Q + q / RX] : E::zero();
                                }
#pragma unroll
                                for (int i = 0; i < RYM; i++) {
                                    const int a = j - i * H;  // kernel row of output row i here
                                    if (i < RY && a >= 0 && a < cky) {
                                        T w[CKX];
                                        load_taps<T, CKX>(w, wsm + (a * S + rho) * TR + t0);
                                        if (!zrow[a]) {
                                            // no zero taps: no per-tap branches (a partial
                                            // chunk in blocks of 8, 4, 2, 1 taps)
                                            if (full) fma_taps<E, RX, 0, CKX>(acc[i], win, w);
                                            else fma_tail<E, RX, CKX / 2, 0>(acc[i], win, w, ckr - t0);
                                        } else {
#pragma unroll
                                            for (int t = 0; t < CKX; t++) {
                                                if (t0 + t < ckr && !E::is_zero(w[t])) {
#pragma unroll
                                                    for (int r = 0; r < RX; r++) E::mac(acc[i][r], win[r + t], w[t]);
                                                }
                                            }
                                        }
                                    }
                                }
                            }
                        }
                    }
                }
            }
        }
    }
    if (warp < nlines) {
#pragma unroll
        for (int i = 0; i < RYM; i++) {
            const int64_t oy = oy0 + ty + (int64_t)i * TY;
            if (i < RY && oy < A1.out) {
                T *yrow = y + oz * P.ys_[0] + oy * P.ys_[1];
#pragma unroll
                for (int r = 0; r < RX; r++) {
                    const int64_t ox = X0 + phi + (int64_t)(sg * SEGW + lane * RX + r) * D;
                    if (ox < A2.out) yrow[ox * P.ys_[2]] = E::out(acc[i][r]);
                }
            }
        }
    }
}

// Output rows a sliding-window line holds at most, per element type (the
// accumulators of RY rows stay in registers).
template <typename T> constexpr int sw_ry_max() { return sizeof(T) <= 4 ? 4 : (sizeof(T) == 8 ? 2 : 1); }

// RYM: rows per line the launch's plan uses (at one row of elements up to
// 8 bytes the accumulators' registers allow three CTAs per SM).
template <typename T, int RX, int CKX, int RYM>
__global__ void __launch_bounds__(256, (RYM == 1 && sizeof(T) <= 8) ? 3 : 2)
    direct_sw_kernel(const T *__restrict__ x0, const T *__restrict__ k0, T *__restrict__ y0,
                     const __grid_constant__ DirectParams<T> P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    direct_sw_block<T, RX, CKX, RYM>(x0, k0, y0, P, blockIdx.x, blockIdx.y, blockIdx.z, smem_raw);
}

// Output o (flat, row-major) of one instance, read through the border map
// with no staging.
template <typename T>
__device__ __forceinline__ void direct_naive_one(const T *__restrict__ x, const T *__restrict__ k,
                                                 T *__restrict__ y, const DirectParams<T> &P, int64_t o) {
    using E = Elem<T>;
    using Acc = typename E::Acc;
    const Geom3<T> &g = P.g;
    const AxisGeom &A0 = g.ax[0], &A1 = g.ax[1], &A2 = g.ax[2];
    const int64_t ox = o % A2.out, oy = (o / A2.out) % A1.out, oz = o / (A2.out * A1.out);
    Acc acc = E::zero();
    for (int64_t kz = P.t_lo[0]; kz < P.t_lo[0] + P.t_n[0]; kz++) {
        const int64_t mz = axis_map(A0, oz * A0.s + kz * A0.d);
        const int64_t kzs = tap_source(kz, A0.K, P.reverse);
        for (int64_t ky = P.t_lo[1]; ky < P.t_lo[1] + P.t_n[1]; ky++) {
            const int64_t my = axis_map(A1, oy * A1.s + ky * A1.d);
            const int64_t kys = tap_source(ky, A1.K, P.reverse);
            for (int64_t kx = P.t_lo[2]; kx < P.t_lo[2] + P.t_n[2]; kx++) {
                const T w = k[kzs * A0.ks + kys * A1.ks + tap_source(kx, A2.K, P.reverse) * A2.ks];
                if (E::is_zero(w)) continue;
                const int64_t mx = axis_map(A2, ox * A2.s + kx * A2.d);
                E::mac(acc, resolve_padded<T>(x, g, mz, my, mx), w);
            }
        }
    }
    y[oz * P.ys_[0] + oy * P.ys_[1] + ox * P.ys_[2]] = E::out(acc);
}

// the persistent batch kernel's naive task: output o if in range
template <typename T> __device__ __forceinline__ void direct_naive_range(const DirectParams<T> &P, int64_t o) {
    const int64_t total = P.g.ax[0].out * P.g.ax[1].out * P.g.ax[2].out;
    if (o < total) direct_naive_one<T>(P.x1, P.k1, P.y1, P, o);
}

// One thread per output.  Used when a tile would not fit in shared memory
// (very large strides); correct for every geometry.
template <typename T>
__global__ void __launch_bounds__(256) direct_naive_kernel(const T *__restrict__ x0,
                                                           const T *__restrict__ k0,
                                                           T *__restrict__ y0, const __grid_constant__ DirectParams<T> P) {
    const int64_t inst = blockIdx.y;
    const T *__restrict__ x = P.xs ? P.xs[P.inst_base + inst] : x0;
    const T *__restrict__ k = P.ks ? P.ks[P.inst_base + inst] : k0;
    T *__restrict__ y = P.ys ? P.ys[P.inst_base + inst] : y0;
    const int64_t total = P.g.ax[0].out * P.g.ax[1].out * P.g.ax[2].out;
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < total;
         o += (int64_t)gridDim.x * blockDim.x)
        direct_naive_one<T>(x, k, y, P, o);
}

// ---- live taps -------------------------------------------------------------
// With every border constant zero, a padded position that does not map to
// an input sample holds zero.  A tap whose positions are such a zero for
// every output contributes 0 * w: exactly nothing for finite w, so the
// kernels loop over the taps [t_lo, t_lo + t_n) that can see data.  If one
// of the skipped weights is Inf or NaN the reference's sums are NaN for
// every output (each output has that tap on a zero); dead_tap_fixup
// reproduces that.
template <typename T> inline bool host_zero(const T &v) { return v == (T)0; }
template <> inline bool host_zero<c32>(const c32 &v) { return v.re == 0.0f && v.im == 0.0f; }
template <> inline bool host_zero<c64>(const c64 &v) { return v.re == 0.0 && v.im == 0.0; }

// Does tap t of an axis (positions t d + o s, o < out) read data (an input
// sample, directly or through the border map) for at least one output?
// The data region [p0, p0 + n) is answered arithmetically; only positions
// in the pads (O(k_eff) of them) consult the border map.
inline bool tap_reads_data(const AxisGeom &A, int64_t t, const std::vector<char> &front,
                           const std::vector<char> &back) {
    const int64_t s = A.s, f = t * A.d, last = f + (A.out - 1) * s;
    const int64_t lo = f > A.p0 ? f : A.p0, hi = last < A.p0 + A.n - 1 ? last : A.p0 + A.n - 1;
    if (lo <= hi) {
        const int64_t p = f + (lo - f + s - 1) / s * s;  // first position >= lo
        if (p <= hi) return true;
    }
    for (int64_t p = f; p <= last && p < A.p0; p += s)
        if (front[(size_t)p]) return true;
    const int64_t b0 = A.p0 + A.n;
    if (last >= b0) {
        int64_t p = f >= b0 ? f : f + (b0 - f + s - 1) / s * s;
        for (; p <= last && p < A.L; p += s)
            if (back[(size_t)(p - b0)]) return true;
    }
    return false;
}

template <typename T> void restrict_live_taps(DirectParams<T> &P) {
    for (int a = 0; a < 3; a++) {
        P.t_lo[a] = 0;
        P.t_n[a] = P.g.ax[a].K;
    }
    for (int a = 0; a < 3; a++)
        if (!host_zero(P.g.cf[a]) || !host_zero(P.g.cb[a])) return;
    int64_t lo[3], n[3];
    for (int a = 0; a < 3; a++) {
        const AxisGeom &A = P.g.ax[a];
        lo[a] = 0;
        n[a] = A.K;
        if (A.K <= 1) continue;
        // pad cells that hold data after the border map
        std::vector<char> front((size_t)(A.p0 > 0 ? A.p0 : 0)), back((size_t)(A.p1 > 0 ? A.p1 : 0));
        for (int64_t j = 0; j < A.p0; j++) front[(size_t)j] = axis_map(A, j) >= 0;
        for (int64_t j = 0; j < A.p1; j++) back[(size_t)j] = axis_map(A, A.p0 + A.n + j) >= 0;
        int64_t first = -1, last = -1;
        for (int64_t t = 0; t < A.K; t++) {
            if (t * A.d >= A.L) break;
            if (tap_reads_data(A, t, front, back)) {
                if (first < 0) first = t;
                last = t;
            }
        }
        if (first < 0) return;  // no tap sees data on this axis: keep the full loops
        lo[a] = first;
        n[a] = last - first + 1;
    }
    for (int a = 0; a < 3; a++) {
        P.t_lo[a] = lo[a];
        P.t_n[a] = n[a];
    }
}

template <typename T> inline bool taps_restricted(const DirectParams<T> &P) {
    for (int a = 0; a < 3; a++)
        if (P.t_lo[a] != 0 || P.t_n[a] != P.g.ax[a].K) return true;
    return false;
}

template <typename T> __device__ __forceinline__ bool non_finite(T v) {
    if constexpr (Elem<T>::kInteger) return false;  // integers are always finite
    else if constexpr (Elem<T>::kComplex) return !isfinite(v.re) || !isfinite(v.im);
    else return !isfinite(v);
}
template <typename T> __device__ __forceinline__ T nan_elem() {
    if constexpr (Elem<T>::kComplex) return T{(decltype(T{}.re))NAN, (decltype(T{}.re))NAN};
    else if constexpr (Elem<T>::kInteger) return T(0);  // not used: integer taps are never non-finite
    else return (T)NAN;
}

// Block-level: scan this block's share of the weights outside the live box;
// if one is not finite, every output of the instance becomes NaN.
template <typename T>
__device__ __forceinline__ void dead_tap_fixup_block(const T *__restrict__ k, T *__restrict__ y,
                                                     const DirectParams<T> &P, int64_t part, int64_t nparts) {
    __shared__ int found;
    if (threadIdx.x == 0) found = 0;
    __syncthreads();
    const AxisGeom &A0 = P.g.ax[0], &A1 = P.g.ax[1], &A2 = P.g.ax[2];
    // kernel rows (ez, ey) split over the parts; within a row whose z and y
    // taps are live only the x taps outside the live range are read
    const int64_t nrows = A0.K * A1.K;
    const int64_t chunk = (nrows + nparts - 1) / nparts;
    const int64_t b = part * chunk, e = (b + chunk < nrows) ? b + chunk : nrows;
    const int64_t lo2 = P.t_lo[2], hi2 = P.t_lo[2] + P.t_n[2];
    bool bad = false;
    for (int64_t r = b + threadIdx.x; r < e; r += blockDim.x) {
        const int64_t ey = r % A1.K, ez = r / A1.K;
        const int64_t ty = tap_source(ey, A1.K, P.reverse), tz = tap_source(ez, A0.K, P.reverse);
        const bool zy_live = tz >= P.t_lo[0] && tz < P.t_lo[0] + P.t_n[0] && ty >= P.t_lo[1] &&
                             ty < P.t_lo[1] + P.t_n[1];
        const T *kr = k + ez * A0.ks + ey * A1.ks;
        if (zy_live) {
            // tap tx is fed by element tap_source(tx) (an involution)
            for (int64_t tx = 0; tx < lo2; tx++) bad |= non_finite(kr[tap_source(tx, A2.K, P.reverse) * A2.ks]);
            for (int64_t tx = hi2; tx < A2.K; tx++) bad |= non_finite(kr[tap_source(tx, A2.K, P.reverse) * A2.ks]);
        } else {
            for (int64_t ex = 0; ex < A2.K; ex++) bad |= non_finite(kr[ex * A2.ks]);
        }
    }
    if (bad) found = 1;
    __syncthreads();
    if (!found) return;
    const int64_t total = A0.out * A1.out * A2.out;
    for (int64_t o = threadIdx.x; o < total; o += blockDim.x) {
        const int64_t ox = o % A2.out, oy = (o / A2.out) % A1.out, oz = o / (A2.out * A1.out);
        y[oz * P.ys_[0] + oy * P.ys_[1] + ox * P.ys_[2]] = nan_elem<T>();
    }
}

namespace direct_detail {
constexpr int kMaxCols = 2048;
constexpr size_t kSmemBudget = 96 * 1024;

template <typename T> size_t smem_bytes(const DirectParams<T> &P) {
    // row maps, column maps, row data offsets, per-row zero-tap flags and
    // per-column staging slots (the last three used by the sliding-window kernel)
    return (size_t)P.maps_off + sizeof(int64_t) * (2 * P.max_rows + P.max_cols) + sizeof(int) * (P.cky + P.max_cols);
}

// Pick block shape and tap chunks so the staged window fits in shared
// memory; returns false when no tile fits (naive kernel then).
template <typename T> bool plan_tile(DirectParams<T> &P, int RX, int &BX, int &BY) {
    const AxisGeom &A1 = P.g.ax[1], &A2 = P.g.ax[2];
    // rows of output per CTA: few when the plane has few rows
    static const int shapes[4][2] = {{32, 8}, {64, 4}, {128, 2}, {256, 1}};
    int pick = 3;
    if (A1.out >= 8) pick = 0;
    else if (A1.out >= 4) pick = 1;
    else if (A1.out >= 2) pick = 2;
    for (; pick < 4; pick++) {
        BX = shapes[pick][0];
        BY = shapes[pick][1];
        const int64_t TX = (int64_t)BX * RX;
        const int64_t base_cols = (TX - 1) * A2.s + 1;
        if (base_cols > kMaxCols) continue;
        int64_t ckx = P.t_n[2];
        if (base_cols + (ckx - 1) * A2.d > kMaxCols) ckx = (kMaxCols - base_cols) / A2.d + 1;
        if (ckx < 1) continue;
        const int64_t W = base_cols + (ckx - 1) * A2.d;
        const int64_t base_rows = (int64_t)(BY - 1) * A1.s + 1;
        // largest cky whose window fits the budget
        int64_t cky = P.t_n[1];
        auto bytes = [&](int64_t c) {
            const int64_t rows = base_rows + (c - 1) * A1.d;
            return sizeof(T) * (rows * W + c * ckx) + 16 + sizeof(int64_t) * (rows + W);
        };
        while (cky > 1 && bytes(cky) > kSmemBudget) cky = (cky + 1) / 2;
        if (bytes(cky) > kSmemBudget) continue;
        P.cky = cky;
        P.ckx = ckx;
        P.max_rows = base_rows + (cky - 1) * A1.d;
        P.max_cols = W;
        P.tile_elems = P.max_rows * W;
        P.w_elems = cky * ckx;
        P.maps_off = ((int64_t)sizeof(T) * (P.tile_elems + P.w_elems) + 15) / 16 * 16;
        P.tile_bx = BX;
        P.tile_by = BY;
        return true;
    }
    return false;
}

inline int64_t gcd64(int64_t a, int64_t b) {
    while (b) {
        const int64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

// Phases D = d / gcd(s, d) and tap residues S = s / gcd(s, d) of the
// contiguous axis; the sliding-window kernel takes D <= 8 and S * D <= 8.
inline bool sw_axis_ok(const AxisGeom &A2, int &D, int &S) {
    const int64_t g = gcd64(A2.s, A2.d);
    const int64_t d = A2.d / g, s = A2.s / g;
    if (d > 8 || s * d > 8) return false;
    D = (int)d;
    S = (int)s;
    return true;
}

// Output columns / rows one sliding-window CTA covers.
template <typename T> inline int64_t sw_cols_per_cta(const DirectParams<T> &P, int RX) {
    return (int64_t)P.sw_nseg * P.sw_ph * 32 * RX;
}
template <typename T> inline int64_t sw_rows_per_cta(const DirectParams<T> &P) {
    return (int64_t)P.sw_ty * P.sw_ry;
}

// Estimated duration (microseconds) of a sliding-window launch over n_inst
// instances, without the per-call overhead (~8.5 us timed from the host:
// planning, launch).  A model whose constants were fitted to GB300 timings
// of every (TY, RY) plan of 620 problems (f32; 1-3-D, 2^8..2^24 elements,
// kernels 3..127 per axis; rms error 14 % of the time):
//  * one warp line: 0.0874 us per window (RX + CKX - 1 shared loads) and
//    0.141 us per (row, kernel row) tap chunk (the FMAs);
//  * the lines of a CTA run concurrently; the SM's issue rate is 0.382 per
//    resident warp line (CTAs per SM: 2, 3 at one row per line, fewer when
//    shared memory is short), at most 4; a CTA holds its slot 4.2 us per
//    staged chunk (global latency, barriers);
//  * one CTA alone takes at least 1.42 x (6.9e-4 us per staged element,
//    its line, 0.037 us per staged chunk).
template <typename T> double sw_time(const DirectParams<T> &P, int RX, int CKX, int64_t n_inst) {
    const AxisGeom &A0 = P.g.ax[0], &A1 = P.g.ax[1], &A2 = P.g.ax[2];
    const int64_t TXo = sw_cols_per_cta(P, RX), TYo = sw_rows_per_cta(P);
    const double ctas = (double)((A2.out + TXo - 1) / TXo) * (double)((A1.out + TYo - 1) / TYo) * (double)A0.out;
    const int S = P.sw_res, D = P.sw_ph, TY = P.sw_ty, RY = P.sw_ry;
    double windows = 0, pairs = 0, staged = 0, chunks = 0;
    const int64_t ny = (P.t_n[1] + P.cky - 1) / P.cky, nx = (P.t_n[2] + P.ckx - 1) / P.ckx;
    for (int64_t iy = 0; iy < ny; iy++) {
        const int64_t cky = iy + 1 < ny ? P.cky : P.t_n[1] - iy * P.cky;
        const double rows = (double)(((int64_t)TY * RY - 1) * A1.s + (cky - 1) * A1.d + 1);
        const double nj = (double)(RY - 1) * P.sw_h + (double)cky;
        for (int64_t ix = 0; ix < nx; ix++) {
            const int64_t ckx = ix + 1 < nx ? P.ckx : P.t_n[2] - ix * P.ckx;
            const int64_t tr0 = (ckx + S - 1) / S;
            staged += rows * (double)S * D * (P.sw_nseg * 32.0 * RX + tr0 - 1);
            chunks += 1;
            for (int r = 0; r < S; r++) {
                const double nch = (double)(((ckx - r + S - 1) / S + CKX - 1) / CKX);  // tap chunks of residue r
                windows += nj * nch;
                pairs += (double)RY * cky * nch;
            }
        }
    }
    const double kz = (double)P.t_n[0];
    const double line = kz * (0.0874 * windows + 0.141 * pairs);
    const double nlines = (double)TY * P.sw_nseg * D;
    const double smem = (double)smem_bytes(P) + 1024.0;
    double resident = (RY == 1 && sizeof(T) <= 8) ? 3.0 : 2.0;
    if (resident * smem > 228.0 * 1024) resident = smem * 2 > 228.0 * 1024 ? 1.0 : 2.0;
    double ipc = 0.382 * resident * nlines;
    if (ipc > 4.0) ipc = 4.0;
    const double spread = ctas * (double)n_inst * (nlines * line / ipc + 4.2 * kz * chunks / resident) / 152.0;
    const double alone = 1.42 * (6.9e-4 * kz * staged + line + 0.037 * kz * chunks);
    return spread > alone ? spread : alone;
}

// Shared-memory layout of a sliding-window plan of TY x RY rows and NSEG
// segments: kernel columns per chunk (all of them when one kernel row fits),
// then kernel rows per chunk.  False when not one tap fits.
template <typename T>
bool sw_layout(DirectParams<T> &P, int RX, int TY, int RY, int H, int NSEG, int D, int S) {
    const AxisGeom &A1 = P.g.ax[1];
    const int SEGW = 32 * RX, CKX = 2 * RX;
    auto geom = [&](int64_t ckx, int64_t cky, int &Q, int64_t &trp, int64_t &rows, int64_t &cols, int64_t &rowe) {
        const int64_t tr = (ckx + S - 1) / S;
        trp = (tr + CKX - 1) / CKX * CKX;  // weight slots: whole tap chunks
        Q = (int)((NSEG * SEGW + tr - 1 + RX - 1) / RX);
        rowe = (int64_t)S * D * RX * Q;
        rows = ((int64_t)TY * RY - 1) * A1.s + (cky - 1) * A1.d + 1;
        cols = (int64_t)S * D * (NSEG * SEGW + tr - 1);
        return sizeof(T) * (rows * rowe + cky * S * trp) + 16 + sizeof(int64_t) * (2 * rows + cols) +
               sizeof(int) * (cky + cols);
    };
    int Q;
    int64_t trp, rows, cols, rowe;
    int64_t ckx = P.t_n[2];
    while (ckx > 1 && geom(ckx, 1, Q, trp, rows, cols, rowe) > kSmemBudget) ckx = (ckx + 1) / 2;
    if (geom(ckx, 1, Q, trp, rows, cols, rowe) > kSmemBudget) return false;
    int64_t cky = P.t_n[1];
    while (cky > 1 && geom(ckx, cky, Q, trp, rows, cols, rowe) > kSmemBudget) cky = (cky + 1) / 2;
    geom(ckx, cky, Q, trp, rows, cols, rowe);
    P.sw_ty = TY;
    P.sw_ry = RY;
    P.sw_h = H;
    P.sw_nseg = NSEG;
    P.sw_q = Q;
    P.sw_ph = D;
    P.sw_res = S;
    P.sw_tr = (int)trp;
    P.cky = cky;
    P.ckx = ckx;
    P.max_rows = rows;
    P.max_cols = cols;
    P.tile_elems = rows * rowe;
    P.w_elems = cky * S * trp;
    P.maps_off = ((int64_t)sizeof(T) * (P.tile_elems + P.w_elems) + 15) / 16 * 16;
    return true;
}

// Sliding-window tiling: warps = TY row sets x NSEG segments x D phases
// (<= 8), RY rows per set.  The first plan is the largest power-of-two TY
// within the warp lines and the output rows (or the autotuner's TY), one row
// per line.  When a kernel row's taps need several chunks, the tap order of
// an output depends on the row chunking, so that plan stays (every launch of
// the problem then sums in one order).  Otherwise all plans give the same
// sums, and the one with the lowest estimated duration for n_inst instances
// is taken among that TY and its half (the best plans of the timed set all
// were) with RY = 1, 2, 4 (RY > 1 where the rows' input rows coincide, i.e.
// TY s1 is a multiple of d1), or with the autotuner's RY.  knobs = false
// ignores the autotuner's settings.
template <typename T> bool plan_sw(DirectParams<T> &P, int RX, int64_t n_inst = 1, bool knobs = true) {
    const AxisGeom &A1 = P.g.ax[1], &A2 = P.g.ax[2];
    int D, S;
    if (!sw_axis_ok(A2, D, S)) return false;
    const int lines = 8 / D;
    const int SEGW = 32 * RX;
    const int64_t segs_needed = (A2.out + (int64_t)D * SEGW - 1) / ((int64_t)D * SEGW);
    auto nseg_for = [&](int ty) {
        int n = lines / ty;
        if (n > segs_needed) n = (int)(segs_needed < 1 ? 1 : segs_needed);
        return n;
    };
    int TY = 1;
    while (TY * 2 <= lines && TY * 2 <= A1.out) TY *= 2;
    // the autotuner's choice of rows per CTA, where it fits the 8 warp lines
    const int want_ty = knobs ? ndconv_tune(NDCONV_TUNE_SW_TY) : 0;
    const bool forced = want_ty > 0 && want_ty <= lines && (want_ty & (want_ty - 1)) == 0;
    if (forced) TY = want_ty;
    if (!sw_layout(P, RX, TY, 1, 0, nseg_for(TY), D, S)) return false;
    if (P.ckx < P.t_n[2]) return true;
    // the autotuner's rows per line (the first plan stays when none fits)
    const int want_ry = knobs ? ndconv_tune(NDCONV_TUNE_SW_RY) : 0;
    const bool ry_forced = want_ry == 1 || want_ry == 2 || want_ry == 4;
    double best = (ry_forced && want_ry != 1) ? 1e300 : sw_time(P, RX, 2 * RX, n_inst);
    DirectParams<T> pick = P;
    const int tys[2] = {TY, (!forced && TY > 1) ? TY / 2 : TY};
    for (int c = 0; c < 2; c++) {
        const int ty = tys[c];
        if (c == 1 && ty == tys[0]) break;
        const bool coincide = ((int64_t)ty * A1.s) % A1.d == 0;
        for (int ry = 1; ry <= sw_ry_max<T>(); ry *= 2) {
            if (ry > 1 && (!coincide || (int64_t)ty * (ry / 2) >= A1.out)) break;
            if ((ty == TY && ry == 1) || (ry_forced && ry != want_ry)) continue;
            DirectParams<T> Q = P;
            const int h = ry > 1 ? (int)((int64_t)ty * A1.s / A1.d) : 0;
            if (!sw_layout(Q, RX, ty, ry, h, nseg_for(ty), D, S) || Q.ckx < Q.t_n[2]) continue;
            const double t = sw_time(Q, RX, 2 * RX, n_inst);
            if (t < best * 0.97) {
                best = t;
                pick = Q;
            }
        }
    }
    P = pick;
    return true;
}

template <typename T, int RX, int CKX>
cudaError_t launch_sw(const T *x, const T *k, T *y, const DirectParams<T> &P, cudaStream_t st, int64_t n_inst) {
    static_assert(CKX % RX == 0, "tap chunks must start on window blocks");
    const size_t sm = smem_bytes(P);
    auto fn = direct_sw_kernel<T, RX, CKX, 1>;
    if constexpr (sw_ry_max<T>() >= 2)
        if (P.sw_ry == 2) fn = direct_sw_kernel<T, RX, CKX, 2>;
    if constexpr (sw_ry_max<T>() >= 4)
        if (P.sw_ry == 4) fn = direct_sw_kernel<T, RX, CKX, 4>;
    cudaError_t e = ndconv_allow_smem((const void *)fn, (int)kSmemBudget + 4096);
    if (e != cudaSuccess) return e;
    const AxisGeom &A0 = P.g.ax[0], &A1 = P.g.ax[1], &A2 = P.g.ax[2];
    const int64_t TXo = sw_cols_per_cta(P, RX);
    const int64_t TYo = sw_rows_per_cta(P);
    dim3 grid((unsigned)((A2.out + TXo - 1) / TXo), (unsigned)((A1.out + TYo - 1) / TYo),
              (unsigned)(A0.out * n_inst));
    fn<<<grid, 256, sm, st>>>(x, k, y, P);
    ndconv_count_launch();
    return cudaGetLastError();
}

template <typename T, int RX> cudaError_t launch_tile(const T *x, const T *k, T *y, const DirectParams<T> &P,
                                                      int BX, int BY, cudaStream_t st, int64_t n_inst) {
    const size_t sm = smem_bytes(P);
    auto fn = direct_tile_kernel<T, RX>;
    cudaError_t e = ndconv_allow_smem((const void *)fn, (int)kSmemBudget + 4096);
    if (e != cudaSuccess) return e;
    const AxisGeom &A0 = P.g.ax[0], &A1 = P.g.ax[1], &A2 = P.g.ax[2];
    const int64_t TX = (int64_t)BX * RX;
    dim3 grid((unsigned)((A2.out + TX - 1) / TX), (unsigned)((A1.out + BY - 1) / BY),
              (unsigned)(A0.out * n_inst));
    fn<<<grid, BX * BY, sm, st>>>(x, k, y, P);
    ndconv_count_launch();
    return cudaGetLastError();
}
}  // namespace direct_detail
using namespace direct_detail;

// Estimated duration (seconds) of a sliding-window launch of one instance, after plan_sw.
template <typename T> double sw_cost(const DirectParams<T> &P, int RX, int CKX) {
    return sw_time(P, RX, CKX, 1) * 1e-6;
}

// With every border constant zero the padded values do not depend on the
// order in which axes are resolved, so the problem may be computed with its
// axes permuted (the output written through permuted strides).  Of the six
// orders, take the one whose sliding-window launch has the lowest estimated
// cost (with the library's own plans, so the tuning knobs never change the
// order, and with it the summation order); when no order fits that kernel, put the longest output axis last
// (the tiled one) and the next longest in the middle.
template <typename T> void permute_axes_for_tiles(DirectParams<T> &P) {
    for (int a = 0; a < 3; a++)
        if (!host_zero(P.g.cf[a]) || !host_zero(P.g.cb[a])) return;
    auto permuted = [&](const int *perm) {
        DirectParams<T> Q = P;
        for (int i = 0; i < 3; i++) {
            Q.g.ax[i] = P.g.ax[perm[i]];
            Q.g.cf[i] = P.g.cf[perm[i]];
            Q.g.cb[i] = P.g.cb[perm[i]];
            Q.t_lo[i] = P.t_lo[perm[i]];
            Q.t_n[i] = P.t_n[perm[i]];
            Q.ys_[i] = P.ys_[perm[i]];
        }
        return Q;
    };
    constexpr int RX = (sizeof(T) <= 4) ? 8 : 4;
    static const int perms[6][3] = {{0, 1, 2}, {1, 0, 2}, {0, 2, 1}, {2, 0, 1}, {1, 2, 0}, {2, 1, 0}};
    double best = 0;
    int pick = -1;
    for (int i = 0; i < 6; i++) {
        DirectParams<T> Q = permuted(perms[i]);
        // the grid's y and z extents are limited to 65535
        if (Q.g.ax[0].out >= 65536 || Q.g.ax[1].out >= 65536) continue;
        if (!plan_sw(Q, RX, 1, false)) continue;
        const double c = sw_cost(Q, RX, 2 * RX);
        if (pick < 0 || c < best * 0.9) {
            best = c;
            pick = i;
        }
    }
    if (pick >= 0) {
        if (pick > 0) P = permuted(perms[pick]);
        return;
    }
    int perm[3] = {0, 1, 2};
    // sort by output extent ascending (stable on ties keeps the original order)
    for (int i = 0; i < 3; i++)
        for (int j = 0; j + 1 < 3 - i; j++)
            if (P.g.ax[perm[j]].out > P.g.ax[perm[j + 1]].out) {
                const int t = perm[j];
                perm[j] = perm[j + 1];
                perm[j + 1] = t;
            }
    if (perm[0] == 0 && perm[1] == 1 && perm[2] == 2) return;
    // do not move a contiguous unit-stride axis away for a longer strided one
    // unless the gain is large (> 4x more outputs)
    if (P.g.ax[perm[2]].out < 4 * P.g.ax[2].out) return;
    P = permuted(perm);
}


}  // namespace ndconv
