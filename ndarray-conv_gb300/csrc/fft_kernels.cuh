// FFT convolution (ConvFFTExt::conv_fft, src/conv_fft/mod.rs:185-292) and
// the FFT processor (src/conv_fft/processor/{real,complex}.rs) on sm_103a.
//
// conv_fft on the canonical 3-axis geometry (axis 2 contiguous):
//   kernel spectrum Kh[F0][F1][H]: row pass over the dilated (optionally
//     flipped) kernel buffer, then column passes over axes 1 and 0;
//   data: row pass (padding evaluated in the load through the border map,
//     zero beyond the padded extent) -> S[P0][F1][H];
//   column pass on axis 1 (3-D only);
//   fused pass on the first non-trivial axis: forward FFT, multiply by Kh,
//     inverse FFT, keep only the rows the crop/stride selects;
//   inverse column pass on axis 1 keeping cropped rows (3-D only);
//   inverse row pass: c2r, scale 1 / prod(F), crop [k_eff-1, pds) step s,
//     write the contiguous output.
// For rank 1 the whole convolution is one fused row kernel.  FFT lengths
// are the smallest 2^a 3^b 5^c 7^d >= pds (even on the real axis): any
// length >= pds gives the same cropped result as the reference's good_size
// (the circular wrap only touches indices < k_eff - 1).
//
// This header holds the row and column pass kernels, their launchers and
// the pass sequence of conv_fft; fft_<type>.cu instantiate the entry points
// per element type and fft_batch.cu the persistent batch kernel.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <mutex>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "fft.h"
#include "fft_core.cuh"

namespace ndconv {

// ------------------------------------------------------------- row pass --
enum RowMode : int {
    ROW_FWD_DATA = 0,    // padded data row -> spectrum row
    ROW_FWD_KERNEL = 1,  // dilated kernel buffer row -> spectrum row
    ROW_INV_OUT = 2,     // spectrum row -> scaled, cropped output row
    ROW_FUSED = 3,       // rank 1: data row -> fwd -> * Kh -> inv -> cropped output
    ROW_FWD_PLAIN = 4,   // contiguous input row -> spectrum row (processor API)
    ROW_INV_PLAIN = 5,   // spectrum row -> scaled contiguous output row (processor API)
    ROW_INV_MAC = 6,     // sum over leading-axis taps of kernel row x data row spectra -> output row
};
enum RowKind : int { RK_COMPLEX = 0, RK_REAL_EVEN = 1, RK_REAL_ODD = 2 };

// One pass over rows of the contiguous axis.  Batched: blockIdx.y selects
// the instance; its data / kernel / output pointers come from the device
// arrays xs / ks / ys (or x / k / y for a single instance) and its spectra
// sit inst * spec_is (kspec_is) elements further.
template <typename T> struct RowArgs {
    using C = typename CplxT<typename Elem<T>::Real>::type;
    using R = typename Elem<T>::Real;
    int mode, kind;
    int64_t F;           // samples per row (real or complex)
    int64_t H;           // spectrum bins per row
    int64_t n_rows, n1;  // row r -> (r / n1, r % n1)
    int64_t spec_s0, spec_s1, spec_is;
    C *spec;
    const C *kspec;
    int64_t kspec_is;
    const T *x;
    Geom3<T> g;
    const T *k;
    int reverse;
    T *y;
    int64_t y_s0, y_s1, out_n, crop_off, crop_step;
    const T *pin;
    T *pout;
    const T *const *xs;
    const T *const *ks;
    T *const *ys;
    int64_t inst_base;
    FftPlanDev pl;   // length M = F/2 (real even) or F
    const C *tw;     // table for pl.L
    const C *twF;    // table for F (real even)
    R scale;
    int nb, lognb;
    // row-spectral form (FFT along the contiguous axis only, taps of the
    // leading axes summed in the spectral domain):
    int kcompact;            // FWD_KERNEL: rows are the K0 x K1 kernel rows in tap order
    int l2only;              // INV_MAC: read spectra through L2 only (same-launch producers)
    int mk0, mk1;            // INV_MAC: leading-axis taps
    int64_t mbase0, mbase1;  // INV_MAC: spectrum offset per output index (stride x row pitch)
    int64_t mstep0, mstep1;  // INV_MAC: spectrum offset per tap (dilation x row pitch)
    int64_t mpitch;          // INV_MAC: row pitch of both spectra (even)
    // INV_MAC grouping (prep_row): a CTA takes nb output rows of one (axis-0
    // index, segment), spaced mac_g apart along axis 1 (residue class c of
    // o1 mod mac_g); mac_gc groups per residue class; mac_win: the group's
    // rows share a register window of data rows (s1 divides d1, spacing d1 / s1)
    int mac_g, mac_win;
    int64_t mac_gc;
    // overlap-save segments along the contiguous axis (seg_n <= 1: whole rows).
    // Row r is (r / seg_n, segment r % seg_n); segment g transforms padded
    // samples [g seg_len, g seg_len + F) and keeps the outputs whose padded
    // position (crop_off + o crop_step) falls in [g seg_len + crop_off,
    // (g + 1) seg_len + crop_off), where the circular sum has no wrap.
    int64_t seg_n, seg_len, spec_sg;
};

// kernel-buffer value at padded position j of one axis: tap index or -1
// (src/conv_fft/padding.rs:78-111: k[i] at i*d, or at k_eff-1-i*d when !reverse)
__device__ __forceinline__ int64_t kbuf_tap(const AxisGeom &a, int64_t j, int reverse) {
    const int64_t q = reverse ? j : (a.keff - 1 - j);
    if (q < 0 || q >= a.keff || q % a.d) return -1;
    return q / a.d;
}

template <typename T> struct RealPart {
    __device__ static typename Elem<T>::Real re(T v) { return v; }
    __device__ static typename Elem<T>::Real im(T) { return 0; }
};
template <> struct RealPart<c32> {
    __device__ static float re(c32 v) { return v.re; }
    __device__ static float im(c32 v) { return v.im; }
};
template <> struct RealPart<c64> {
    __device__ static double re(c64 v) { return v.re; }
    __device__ static double im(c64 v) { return v.im; }
};

template <typename T> __device__ __forceinline__ T make_elem(typename Elem<T>::Real re, typename Elem<T>::Real im) {
    if constexpr (Elem<T>::kComplex) return T{re, im};
    else return (T)re;
}

// per-row facts shared by the CTA
struct RowInfo {
    int64_t xoff;    // data: offset of the row's first input sample (interior rows)
    int64_t soff;    // spectrum row offset
    int64_t yoff;    // output row offset
    int64_t m0, m1;  // data: border-mapped leading indices
    int64_t t0, t1;  // kernel: tap indices of the leading axes (-1: zero row)
    int64_t j0;      // padded position of the segment's first sample
    int o_lo, o_hi;  // outputs [o_lo, o_hi) of the row come from this segment
    int valid, interior;
};

// sample j of a row for the forward loads (MODE is the RowMode)
template <int MODE, typename T>
__device__ __forceinline__ T row_sample(const RowArgs<T> &A, const T *__restrict__ x, const T *__restrict__ k,
                                        const RowInfo &ri, int64_t row, int64_t j) {
    if constexpr (MODE == ROW_FWD_PLAIN) {
        return A.pin[row * A.F + j];
    } else if constexpr (MODE == ROW_FWD_KERNEL) {
        if (ri.t0 < 0 || ri.t1 < 0) return Elem<T>::zero();
        const int64_t t2 = kbuf_tap(A.g.ax[2], j, A.reverse);
        if (t2 < 0) return Elem<T>::zero();
        return k[ri.t0 * A.g.ax[0].ks + ri.t1 * A.g.ax[1].ks + t2 * A.g.ax[2].ks];
    } else {
        // data (FWD_DATA / FUSED): zero beyond the padded extent
        const AxisGeom &a2 = A.g.ax[2];
        j += ri.j0;
        if (ri.interior && j >= a2.p0 && j < a2.p0 + a2.n) return x[ri.xoff + (j - a2.p0) * a2.xs];
        if (j >= a2.L) return Elem<T>::zero();
        return resolve_padded<T>(x, A.g, ri.m0, ri.m1, axis_map(a2, j));
    }
}

// Asynchronous global -> shared copies (cp.async, completed by
// cp_async_wait_all): a row's interior samples are all in flight at once
// and never pass through registers.  BYTES is 4, 8 or 16; both addresses
// are aligned to it.
template <int BYTES> __device__ __forceinline__ void cp_async(void *smem, const void *gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(sa), "l"(gmem), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// r2c post-processing of one bin: X[k] from a = Z[k mod M] and c = Z[(M - k) mod M]
// of Z = FFT_M(x[2m] + i x[2m+1]): X[k] = E + w (-i D), E = (a + conj c) / 2,
// D = (a - conj c) / 2, w = exp(-2 pi i k / 2M).
template <typename C> __device__ __forceinline__ C r2c_bin(C a, C c, C w) {
    using R = decltype(a.re);
    c = cconj(c);
    const C e = C{(R)0.5 * (a.re + c.re), (R)0.5 * (a.im + c.im)};
    const C d = C{(R)0.5 * (a.re - c.re), (R)0.5 * (a.im - c.im)};
    const C o = C{d.im, -d.re};  // -i * d
    const C wo = cmul(w, o);
    return C{e.re + wo.re, e.im + wo.im};
}

// c2r pre-processing of one bin: Z[k] (k < M) from a = X[k] and c = X[M - k]
// of a Hermitian spectrum X[0..M], such that IFFT_M(Z)[j] = x[2j] + i x[2j+1]
// for the unnormalised length-2M inverse (imaginary parts of the DC and
// Nyquist bins ignored: k0 marks k = 0).
template <typename C> __device__ __forceinline__ C c2r_bin(C a, C c, C w, bool k0) {
    if (k0) {
        a.im = 0;
        c.im = 0;
    }
    c = cconj(c);
    const C e = cadd(a, c);
    const C d = csub(a, c);
    const C o = cmul(d, cconj(w));
    return C{e.re - o.im, e.im + o.re};  // e + i*o
}

// mirror bin of k in a real row's spectrum X[0..M]: M - k (k = 0: the Nyquist bin M)
__device__ __forceinline__ int mirror_bin(int k, int M) { return k == 0 ? M : M - k; }

// complex multiply-add in the order every spectral tap sum uses
template <typename C> __device__ __forceinline__ C cfma(C k, C d, C acc) {
    acc.re = fmaf_t(k.re, d.re, fmaf_t(-k.im, d.im, acc.re));
    acc.im = fmaf_t(k.re, d.im, fmaf_t(k.im, d.re, acc.im));
    return acc;
}

// Spectral tap sum of a group of nb output rows (ROW_INV_MAC).  For every
// bin, row b's sum runs over the leading taps (tz, ty) in ascending order
// (tz outer) of Kh[tz][ty] x S[data row of (b, tz, ty)], so the result does
// not depend on how rows are grouped.  Real rows of even length (PAIR) take
// bins k and M - k together and leave the c2r pre-processed Z[k], Z[M - k]
// in Z; other kinds leave the bins as they are.  With A.mac_win the group's
// rows are spaced d1 / s1 apart along axis 1, so row b + 1 at tap ty reads
// the data row of row b at tap ty + 1: NR rows at a time share one register
// window of data rows, each loaded once per tap of axis 0.  A thread takes
// U units (bins, or bin pairs) 32 apart, so that their loads share one
// address per spectrum row.
template <typename T, bool PAIR, int NR, int U, typename Load>
__device__ __forceinline__ void mac_group(const RowArgs<T> &A, const typename RowArgs<T>::C *__restrict__ kspec,
                                          const typename RowArgs<T>::C *__restrict__ spec, const RowInfo *rinfo,
                                          typename RowArgs<T>::C *Z, int M, int H, int nb, int lognb, Load load) {
    using C = typename RowArgs<T>::C;
    const int mk0 = A.mk0, mk1 = A.mk1;
    const int64_t st0 = A.mstep0, st1 = A.mstep1, Hh = A.mpitch;
    const int nunits = PAIR ? (M >> 1) + 1 : H;
    const AxisGeom &a1 = A.g.ax[1];
    const C zero = C{0, 0};
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int rb = 0; rb < nb; rb += NR) {
        const RowInfo &r0 = rinfo[rb];
        if (!r0.valid) break;  // rows of a group are in ascending order: the rest are invalid too
        // window slots s whose data row o1 s1 + s d1 lies inside the padded axis
        int nslot = 0;
        if (A.mac_win) {
            const int64_t top = a1.L - 1 - r0.m1 * a1.s;
            nslot = top < 0 ? 0 : (int)min((int64_t)(NR + mk1), top / a1.d + 1);
        }
        for (int k0 = warp * 32 * U + lane; k0 < nunits; k0 += nwarps * 32 * U) {
            bool ok[U];
#pragma unroll
            for (int u = 0; u < U; u++) ok[u] = k0 + 32 * u < nunits;
            // bin k of unit u: k0 + 32 u; its mirror M - k0 - 32 u (k = 0: bin M)
            C acc0[U][NR], acc1[U][NR];
#pragma unroll
            for (int u = 0; u < U; u++)
#pragma unroll
                for (int b = 0; b < NR; b++) acc0[u][b] = acc1[u][b] = zero;
            for (int tz = 0; tz < mk0; tz++) {
                const C *pk = kspec + (int64_t)tz * mk1 * Hh + k0;
                const C *pkm = kspec + (int64_t)tz * mk1 * Hh + (M - k0);
                if (A.mac_win) {
                    const C *pd = spec + r0.soff + tz * st0 + k0;
                    const C *pdm = spec + r0.soff + tz * st0 + (M - k0);
                    C d0[U][NR], d1[U][NR];
#pragma unroll
                    for (int sl = 0; sl < NR - 1; sl++) {
                        const bool v = sl < nslot;
#pragma unroll
                        for (int u = 0; u < U; u++) {
                            d0[u][sl] = (v && ok[u]) ? load(pd + 32 * u) : zero;
                            if constexpr (PAIR) d1[u][sl] = (v && ok[u]) ? load(pdm - 32 * u) : zero;
                        }
                        pd += st1;
                        pdm += st1;
                    }
                    for (int ty = 0; ty < mk1; ty++) {
                        const bool v = NR - 1 + ty < nslot;
#pragma unroll
                        for (int u = 0; u < U; u++) {
                            d0[u][NR - 1] = (v && ok[u]) ? load(pd + 32 * u) : zero;
                            if constexpr (PAIR) d1[u][NR - 1] = (v && ok[u]) ? load(pdm - 32 * u) : zero;
                            const C k0v = ok[u] ? load(pk + 32 * u) : zero;
#pragma unroll
                            for (int b = 0; b < NR; b++) acc0[u][b] = cfma(k0v, d0[u][b], acc0[u][b]);
                            if constexpr (PAIR) {
                                const C k1v = ok[u] ? load(pkm - 32 * u) : zero;
#pragma unroll
                                for (int b = 0; b < NR; b++) acc1[u][b] = cfma(k1v, d1[u][b], acc1[u][b]);
                            }
#pragma unroll
                            for (int b = 0; b < NR - 1; b++) {
                                d0[u][b] = d0[u][b + 1];
                                if constexpr (PAIR) d1[u][b] = d1[u][b + 1];
                            }
                        }
                        pd += st1;
                        pdm += st1;
                        pk += Hh;
                        pkm += Hh;
                    }
                } else {
                    for (int ty = 0; ty < mk1; ty++) {
#pragma unroll
                        for (int u = 0; u < U; u++) {
                            const C k0v = ok[u] ? load(pk + 32 * u) : zero;
                            C k1v = zero;
                            if constexpr (PAIR) k1v = ok[u] ? load(pkm - 32 * u) : zero;
#pragma unroll
                            for (int b = 0; b < NR; b++) {
                                const RowInfo &ri = rinfo[rb + b];
                                if (!ri.valid || !ok[u]) continue;
                                const C *sp = spec + ri.soff + tz * st0 + ty * st1;
                                acc0[u][b] = cfma(k0v, load(sp + k0 + 32 * u), acc0[u][b]);
                                if constexpr (PAIR) acc1[u][b] = cfma(k1v, load(sp + (M - k0) - 32 * u), acc1[u][b]);
                            }
                        }
                        pk += Hh;
                        pkm += Hh;
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (!ok[u]) continue;
                const int k = k0 + 32 * u, km = M - k;
#pragma unroll
                for (int b = 0; b < NR; b++) {
                    if constexpr (PAIR) {
                        Z[sx<C>((k << lognb) + rb + b)] = c2r_bin(acc0[u][b], acc1[u][b], ldg_c(A.twF + k), k == 0);
                        if (k != 0 && km != k)
                            Z[sx<C>((km << lognb) + rb + b)] = c2r_bin(acc1[u][b], acc0[u][b], ldg_c(A.twF + km), false);
                    } else {
                        Z[sx<C>((k << lognb) + rb + b)] = acc0[u][b];
                    }
                }
            }
        }
    }
}

// One CTA's share of a row pass: rows [bx * nb, bx * nb + nb) of instance by
// (ROW_INV_MAC: the group of nb output rows bx, see prep_row).
// The row transform: the compile-time geometry for a specialised length FL
// (FNB rows per CTA), else the run-time one.
template <bool INV, int FL, int FNB, typename C>
__device__ __forceinline__ C *row_fft(C *a, C *b, int nb, int lognb, const FftPlanDev &pl, const C *tw) {
    if constexpr (FL == 2560) return block_fft_ct<INV, 2560, FNB, 16, 16, 10>(a, b, pl);
    else return block_fft<INV>(a, b, nb, lognb, pl, tw);
}

// Lengths whose row transforms are specialised at compile time (their plan
// must be the one make_plan gives them): 2560-point complex transforms, the
// 5120-sample real rows of the benchmark cases, in CTAs of one or two rows.
// Same arithmetic as the run-time path; only the index computations fold.
template <typename T> __device__ __forceinline__ int fixed_rows(const RowArgs<T> &A) {
    if constexpr (std::is_same<T, float>::value) {
        if (A.pl.L == 2560 && A.pl.nst == 3 && (A.nb == 1 || A.nb == 2)) return A.nb;
    }
    return 0;
}

template <typename T, int MODE, int FL = 0, int FNB = 0>
__device__ __forceinline__ void row_block(const RowArgs<T> &A, unsigned bx, unsigned by, unsigned char *smem_raw) {
    using C = typename RowArgs<T>::C;
    using R = typename RowArgs<T>::R;
    const int nb = FL ? FNB : A.nb, lognb = FL ? (FNB == 2 ? 1 : 0) : A.lognb;
    const int M = FL ? FL : A.pl.L;  // transform length
    const int cap = (int)padded_slots<C>((int64_t)(A.kind == RK_REAL_EVEN ? M + 1 : M) << lognb);
    RowInfo *rinfo = reinterpret_cast<RowInfo *>(smem_raw);
    C *buf0 = reinterpret_cast<C *>(smem_raw + ((sizeof(RowInfo) * nb + 15) / 16) * 16);
    C *buf1 = buf0 + cap;
    const int inst = (int)by;
    const T *__restrict__ x = A.xs ? A.xs[A.inst_base + inst] : A.x;
    const T *__restrict__ kp = A.ks ? A.ks[A.inst_base + inst] : A.k;
    T *__restrict__ y = A.ys ? A.ys[A.inst_base + inst] : A.y;
    C *spec = A.spec + inst * A.spec_is;
    const C *kspec = A.kspec + inst * A.kspec_is;
    const int64_t rbase = (int64_t)bx * nb;
    const int64_t sn = A.seg_n > 1 ? A.seg_n : 1;

    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        RowInfo ri{};
        int64_t i0, i1, seg;
        if constexpr (MODE == ROW_INV_MAC) {
            // group bx = (outer, residue c, group): rows o1 = c + g (group nb + b)
            const int64_t gg = A.mac_g, gc = A.mac_gc;
            const int64_t outer = (int64_t)bx / (gg * gc), rem = (int64_t)bx - outer * gg * gc;
            const int64_t c = rem / gc, grp = rem - c * gc;
            i0 = outer / sn;
            seg = outer - i0 * sn;
            i1 = c + gg * (grp * nb + b);
            ri.valid = i1 < A.n1;
            ri.m1 = i1;
        } else {
            const int64_t r = rbase + b;
            const int64_t rr = r / sn;
            seg = r - rr * sn;
            i0 = rr / A.n1;
            i1 = rr - i0 * A.n1;
            ri.valid = r < A.n_rows;
        }
        ri.soff = i0 * A.spec_s0 + i1 * A.spec_s1 + seg * A.spec_sg;
        ri.yoff = i0 * A.y_s0 + i1 * A.y_s1;
        if (sn > 1) {
            const int64_t cs = A.crop_step;
            ri.j0 = seg * A.seg_len;
            ri.o_lo = (int)((seg * A.seg_len + cs - 1) / cs);
            ri.o_hi = (int)min(A.out_n, ((seg + 1) * A.seg_len + cs - 1) / cs);
        } else {
            ri.j0 = 0;
            ri.o_lo = 0;
            ri.o_hi = (int)A.out_n;
        }
        if constexpr (MODE == ROW_FWD_DATA || MODE == ROW_FUSED) {
            ri.m0 = axis_map(A.g.ax[0], i0);
            ri.m1 = axis_map(A.g.ax[1], i1);
            ri.interior = ri.m0 >= 0 && ri.m1 >= 0;
            ri.xoff = ri.interior ? ri.m0 * A.g.ax[0].xs + ri.m1 * A.g.ax[1].xs : 0;
        } else if constexpr (MODE == ROW_FWD_KERNEL) {
            if (A.kcompact) {
                ri.t0 = tap_source(i0, A.g.ax[0].K, A.reverse);
                ri.t1 = tap_source(i1, A.g.ax[1].K, A.reverse);
            } else {
                ri.t0 = kbuf_tap(A.g.ax[0], i0, A.reverse);
                ri.t1 = kbuf_tap(A.g.ax[1], i1, A.reverse);
            }
        } else if constexpr (MODE == ROW_INV_MAC) {
            ri.soff = i0 * A.mbase0 + i1 * A.mbase1 + seg * A.spec_sg;
        }
        rinfo[b] = ri;
    }
    __syncthreads();
    // blockDim is a multiple of nb, so a thread always works on the same row
    // b = tid mod nb of the CTA: its row facts live in registers
    const int bt = threadIdx.x & (nb - 1);
    const RowInfo rit = rinfo[bt];

    constexpr bool fwd = (MODE == ROW_FWD_DATA || MODE == ROW_FWD_KERNEL || MODE == ROW_FUSED ||
                          MODE == ROW_FWD_PLAIN);
    const bool pair = (A.kind == RK_REAL_EVEN);
    C *res;
    if constexpr (fwd) {
        // ---- load samples: element (b, i) -> buf0[i * nb + b], four independent loads per round
        const int total = M << lognb;
        const int T_ = blockDim.x;
        // interior samples of a data row (contiguous axis of unit stride) by
        // plain loads: padded positions [lo, hi) of the row's window are
        // x[xb + j]; sample pairs load as one vector when aligned
        bool fastrow = false;
        int64_t xb = 0;
        int lo = 0, hi = 0;
        bool vec2 = false;
        if constexpr (MODE == ROW_FWD_DATA || MODE == ROW_FUSED) {
            const AxisGeom &a2 = A.g.ax[2];
            if (pair && a2.xs == 1 && rit.interior) {
                fastrow = true;
                xb = rit.xoff + rit.j0 - a2.p0;
                lo = (int)max((int64_t)0, a2.p0 - rit.j0);
                hi = (int)min((int64_t)2 * M, a2.p0 + a2.n - rit.j0);
                vec2 = ((reinterpret_cast<uintptr_t>(x) + (uintptr_t)(xb * (int64_t)sizeof(T))) % (2 * sizeof(T))) == 0;
            }
        }
        for (int u0 = threadIdx.x; u0 < total; u0 += 4 * T_) {
            C v[4];
            bool async[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int u = u0 + q * T_;
                v[q] = C{0, 0};
                async[q] = false;
                if (u < total && rit.valid) {
                    const int i = u >> lognb;
                    const int64_t r = rbase + bt;
                    if (pair) {
                        const int j = 2 * i;
                        if (fastrow && j >= lo && j + 1 < hi) {
                            // interior sample pair: straight into shared memory
                            if constexpr (!Elem<T>::kComplex) {
                                T *d = reinterpret_cast<T *>(&buf0[sx<C>(u)]);
                                if (vec2) {
                                    cp_async<2 * sizeof(T)>(d, x + xb + j);
                                } else {
                                    cp_async<sizeof(T)>(d, x + xb + j);
                                    cp_async<sizeof(T)>(d + 1, x + xb + j + 1);
                                }
                                async[q] = true;
                            }
                        } else {
                            const T s0 = row_sample<MODE>(A, x, kp, rit, r, (int64_t)j);
                            const T s1 = row_sample<MODE>(A, x, kp, rit, r, (int64_t)j + 1);
                            v[q] = C{RealPart<T>::re(s0), RealPart<T>::re(s1)};
                        }
                    } else {
                        const T sm = row_sample<MODE>(A, x, kp, rit, r, i);
                        v[q] = C{RealPart<T>::re(sm), RealPart<T>::im(sm)};
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int u = u0 + q * T_;
                if (u < total && !async[q]) buf0[sx<C>(u)] = v[q];
            }
        }
        if (fastrow) cp_async_wait_all();
        __syncthreads();
        res = row_fft<false, FL, FNB>(buf0, buf1, nb, lognb, A.pl, A.tw);
        C *other = (res == buf0) ? buf1 : buf0;
        const int H = (int)A.H;
        if constexpr (MODE != ROW_FUSED) {
            if (pair) {
                // r2c post-processing straight into the spectrum rows: bins k and M - k
                const int tot = ((M >> 1) + 1) << lognb;
                if (rit.valid)
                    for (int u = threadIdx.x; u < tot; u += blockDim.x) {
                        const int k = u >> lognb, km = mirror_bin(k, M);
                        const C z0 = res[sx<C>(((k == 0 ? 0 : k) << lognb) + bt)];
                        const C z1 = res[sx<C>(((k == 0 ? 0 : km) << lognb) + bt)];
                        spec[rit.soff + k] = r2c_bin(z0, z1, ldg_c(A.twF + k));
                        if (km != k) spec[rit.soff + km] = r2c_bin(z1, z0, ldg_c(A.twF + km));
                    }
            } else {
                const int tot = H << lognb;
                if (rit.valid)
                    for (int u = threadIdx.x; u < tot; u += blockDim.x) spec[rit.soff + (u >> lognb)] = res[sx<C>(u)];
            }
            return;
        }
        // ---- fused: multiply by the kernel spectrum, back to the time domain
        if (pair) {
            // post-process, multiply and pre-process bins k and M - k in place
            const int tot = ((M >> 1) + 1) << lognb;
            for (int u = threadIdx.x; u < tot; u += blockDim.x) {
                const int k = u >> lognb, km = mirror_bin(k, M);
                const int s0 = sx<C>(((k == 0 ? 0 : k) << lognb) + bt);
                const int s1 = sx<C>(((k == 0 ? 0 : km) << lognb) + bt);
                const C z0 = res[s0], z1 = res[s1];
                const C x0 = cmul(r2c_bin(z0, z1, ldg_c(A.twF + k)), ldcg_c(kspec + k));
                const C x1 = cmul(r2c_bin(z1, z0, ldg_c(A.twF + km)), ldcg_c(kspec + km));
                res[s0] = c2r_bin(x0, x1, ldg_c(A.twF + k), k == 0);
                if (k != 0 && km != k) res[s1] = c2r_bin(x1, x0, ldg_c(A.twF + km), false);
            }
            __syncthreads();
            res = row_fft<true, FL, FNB>(res, other, nb, lognb, A.pl, A.tw);
        } else {
            const int tot = H << lognb;
            for (int u = threadIdx.x; u < tot; u += blockDim.x) res[sx<C>(u)] = cmul(res[sx<C>(u)], ldcg_c(kspec + (u >> lognb)));
            __syncthreads();
            res = row_fft<true, FL, FNB>(res, other, nb, lognb, A.pl, A.tw);
        }
    } else {
        // ---- inverse: spectrum rows (real rows of even length: c2r
        // pre-processed on the way in) into buf0
        const int H = (int)A.H;
        if constexpr (MODE == ROW_INV_MAC) {
            const int nr = nb < 4 ? nb : 4;
            auto run = [&](auto load) {
                // one unit per thread: measured on 2560-point rows in groups of two,
                // two units 32 apart ran 10 % slower (fewer warps share the units)
                if (pair) {
                    if (nr == 1) mac_group<T, true, 1, 1>(A, kspec, spec, rinfo, buf0, M, H, nb, lognb, load);
                    else if (nr == 2) mac_group<T, true, 2, 1>(A, kspec, spec, rinfo, buf0, M, H, nb, lognb, load);
                    else mac_group<T, true, 4, 1>(A, kspec, spec, rinfo, buf0, M, H, nb, lognb, load);
                } else {
                    if (nr == 1) mac_group<T, false, 1, 1>(A, kspec, spec, rinfo, buf0, M, H, nb, lognb, load);
                    else if (nr == 2) mac_group<T, false, 2, 1>(A, kspec, spec, rinfo, buf0, M, H, nb, lognb, load);
                    else mac_group<T, false, 4, 1>(A, kspec, spec, rinfo, buf0, M, H, nb, lognb, load);
                }
            };
            // the load kind is uniform: one loop nest per kind, no per-load select
            if (A.l2only) run([](const C *p) { return ldcg_c(p); });
            else run([](const C *p) { return ldg_c(p); });
        } else if (pair) {
            const int tot = ((M >> 1) + 1) << lognb;
            for (int u = threadIdx.x; u < tot; u += blockDim.x) {
                const int k = u >> lognb, km = mirror_bin(k, M);
                const C x0 = rit.valid ? ldcg_c(spec + rit.soff + k) : C{0, 0};
                const C x1 = rit.valid ? ldcg_c(spec + rit.soff + km) : C{0, 0};
                buf0[sx<C>((k << lognb) + bt)] = c2r_bin(x0, x1, ldg_c(A.twF + k), k == 0);
                if (k != 0 && km != k) buf0[sx<C>((km << lognb) + bt)] = c2r_bin(x1, x0, ldg_c(A.twF + km), false);
            }
        } else {
            const int tot = H << lognb;
            for (int u = threadIdx.x; u < tot; u += blockDim.x)
                buf0[sx<C>(u)] = rit.valid ? ldcg_c(spec + rit.soff + (u >> lognb)) : C{0, 0};
        }
        __syncthreads();
        if (A.kind == RK_REAL_ODD) {
            // Hermitian extension to the full length (DC imaginary part ignored)
            const int tot2 = M << lognb;
            for (int u = threadIdx.x; u < tot2; u += blockDim.x) {
                const int b = u & (nb - 1), k = u >> lognb;
                if (k >= H) buf0[sx<C>(u)] = cconj(buf0[sx<C>(((M - k) << lognb) + b)]);
                else if (k == 0) buf0[sx<C>(u)].im = 0;
            }
            __syncthreads();
        }
        res = row_fft<true, FL, FNB>(buf0, buf1, nb, lognb, A.pl, A.tw);
    }
    // ---- store time-domain samples (scaled; cropped + strided for INV_OUT / FUSED)
    constexpr bool plain = (MODE == ROW_INV_PLAIN);
    const bool segs = !plain && A.seg_n > 1;
    // outputs per row (per segment: at most ceil(seg_len / crop_step))
    const int n_out = (int)(plain ? A.F : segs ? (A.seg_len + A.crop_step - 1) / A.crop_step : A.out_n);
    const int tot = n_out << lognb;
    // the row's output facts are read back from shared memory here rather
    // than kept in registers through the transforms and the tap sums
    const RowInfo &ri = rinfo[bt];
    const int coff = (int)(A.crop_off - ri.j0), cstep = (int)A.crop_step;
    if (!ri.valid) return;
    for (int u = threadIdx.x; u < tot; u += blockDim.x) {
        const int b = bt;
        const int o = plain ? (u >> lognb) : ri.o_lo + (u >> lognb);
        if (!plain && o >= ri.o_hi) continue;
        const int p = plain ? o : (coff + o * cstep);
        R vr, vi;
        if (A.kind == RK_REAL_EVEN) {
            const C z = res[sx<C>(((p >> 1) << lognb) + b)];
            vr = (p & 1) ? z.im : z.re;
            vi = 0;
        } else {
            const C z = res[sx<C>((p << lognb) + b)];
            vr = z.re;
            vi = z.im;
        }
        const T v = make_elem<T>(vr * A.scale, vi * A.scale);
        if constexpr (plain) A.pout[(rbase + b) * A.F + o] = v;
        else y[ri.yoff + o] = v;
    }
}

// MAXT 512 caps registers at 64 (4 CTAs of 256 threads per SM: launches of
// many CTAs, throughput-bound); MAXT 384 allows 85, so that a launch of few
// CTAs (latency-bound, at most two per SM) keeps more values in registers
// instead of spilling.
template <typename T, int MODE, int MAXT>
__global__ void __launch_bounds__(MAXT, 2) row_kernel(const __grid_constant__ RowArgs<T> A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    if constexpr (std::is_same<T, float>::value && MODE != ROW_FWD_PLAIN && MODE != ROW_INV_PLAIN) {
        const int f = fixed_rows(A);
        if (f == 1) return row_block<T, MODE, 2560, 1>(A, blockIdx.x, blockIdx.y, smem_raw);
        if (f == 2) return row_block<T, MODE, 2560, 2>(A, blockIdx.x, blockIdx.y, smem_raw);
    }
    row_block<T, MODE>(A, blockIdx.x, blockIdx.y, smem_raw);
}

// ---------------------------------------------------------- column pass --
enum ColMode : int { COL_FWD = 0, COL_INV = 1, COL_FUSED = 2 };

// One pass over a strided axis: columns [h0, h0 + nb) of the contiguous
// inner extent, outer index blockIdx.y (grid-strided), instance blockIdx.z
// (buffers inst * src_is / dst_is / k_is elements further).
template <typename C> struct ColArgs {
    int mode;
    const C *src;
    C *dst;
    int64_t n_inner, n_outer;
    int64_t src_outer, src_axis, dst_outer, dst_axis;
    int64_t src_is, dst_is;
    int64_t valid_in;
    int64_t crop_off, crop_step, n_out;
    const C *kspec;
    int64_t k_axis, k_is;
    FftPlanDev pl;
    const C *tw;
    int nb, lognb;
};

// One CTA's share of a column pass: column tile bx, outer indices by,
// by + ystep, ... of instance bz.
template <typename C>
__device__ __forceinline__ void col_block(const ColArgs<C> &A, unsigned bx, int64_t by, int64_t ystep, unsigned bz,
                                          unsigned char *smem_raw) {
    const int nb = A.nb, lognb = A.lognb;
    const int F = A.pl.L;
    C *buf0 = reinterpret_cast<C *>(smem_raw);
    C *buf1 = buf0 + padded_slots<C>((int64_t)F << lognb);
    const int64_t h0 = (int64_t)bx * nb;
    const int inst = (int)bz;
    const int nvalid = (int)(h0 + nb <= A.n_inner ? nb : A.n_inner - h0);
    const int valid_in = (int)A.valid_in;
    const int T_ = blockDim.x;
    for (int64_t outer = by; outer < A.n_outer; outer += ystep) {
        const C *__restrict__ src = A.src + inst * A.src_is + outer * A.src_outer + h0;
        const int tot_in = F << lognb;
        for (int u0 = threadIdx.x; u0 < tot_in; u0 += 4 * T_) {
            C v[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int u = u0 + q * T_;
                const int b = u & (nb - 1), i = u >> lognb;
                v[q] = C{0, 0};
                if (u < tot_in && i < valid_in && b < nvalid) v[q] = ldcg_c(src + i * A.src_axis + b);
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int u = u0 + q * T_;
                if (u < tot_in) buf0[sx<C>(u)] = v[q];
            }
        }
        __syncthreads();
        C *res;
        if (A.mode == COL_INV) {
            res = block_fft<true>(buf0, buf1, nb, lognb, A.pl, A.tw);
        } else {
            res = block_fft<false>(buf0, buf1, nb, lognb, A.pl, A.tw);
            if (A.mode == COL_FUSED) {
                const C *__restrict__ kp = A.kspec + inst * A.k_is + h0;
                for (int u = threadIdx.x; u < tot_in; u += T_) {
                    const int b = u & (nb - 1), k = u >> lognb;
                    if (b < nvalid) res[sx<C>(u)] = cmul(res[sx<C>(u)], ldcg_c(kp + k * A.k_axis + b));
                }
                __syncthreads();
                C *other = (res == buf0) ? buf1 : buf0;
                res = block_fft<true>(res, other, nb, lognb, A.pl, A.tw);
            }
        }
        C *dst = A.dst + inst * A.dst_is + outer * A.dst_outer + h0;
        const int n_out = (A.mode == COL_FWD) ? F : (int)A.n_out;
        const int tot_out = n_out << lognb;
        const int coff = (int)A.crop_off, cstep = (int)A.crop_step;
        for (int u = threadIdx.x; u < tot_out; u += T_) {
            const int b = u & (nb - 1), o = u >> lognb;
            if (b >= nvalid) continue;
            const int p = (A.mode == COL_FWD) ? o : (coff + o * cstep);
            dst[o * A.dst_axis + b] = res[sx<C>((p << lognb) + b)];
        }
        __syncthreads();
    }
}

template <typename C>
__global__ void __launch_bounds__(256, 2) col_kernel(const __grid_constant__ ColArgs<C> A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    col_block<C>(A, blockIdx.x, blockIdx.y, gridDim.y, blockIdx.z, smem_raw);
}

// ----------------------------------------------------------- transpose --
template <typename C>
__global__ void transpose_kernel(const C *__restrict__ in, C *__restrict__ out, int64_t rows, int64_t cols) {
    __shared__ C tile[32][33];
    const int64_t c0 = (int64_t)blockIdx.x * 32, r0 = (int64_t)blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int64_t r = r0 + i, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[i][threadIdx.x] = in[r * cols + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int64_t c = c0 + i, r = r0 + threadIdx.x;
        if (r < rows && c < cols) out[c * rows + r] = tile[threadIdx.x][i];
    }
}

// ------------------------------------------------------------- launchers --
namespace {
constexpr int kThreads = 256;
constexpr size_t kFftSmemMax = 200 * 1024;
constexpr size_t kSmemPerSm = 228 * 1024;  // shared memory of one SM
constexpr int64_t kFewCtas = 4 * 152;  // launches up to this many CTAs are latency-bound
constexpr int kFewThreads = 384;        // their widest CTA

int ilog2(int v) {
    int l = 0;
    while ((1 << l) < v) l++;
    return l;
}

template <typename K> int ensure_smem(K fn) {
    const cudaError_t e = ndconv_allow_smem((const void *)fn, (int)kFftSmemMax);
    if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
    return NDCONV_OK;
}

template <typename T> size_t row_smem(const RowArgs<T> &A) {
    using C = typename RowArgs<T>::C;
    const int64_t cap = padded_slots<C>((A.kind == RK_REAL_EVEN ? A.pl.L + 1 : A.pl.L) * A.nb);
    return ((sizeof(RowInfo) * A.nb + 15) / 16) * 16 + sizeof(C) * 2 * cap;
}

// rows per CTA: enough to give each CTA ~2K samples, at least 1
int pick_nb(int64_t len, int64_t rows, size_t per_row_bytes, size_t cap) {
    int nb = 1;
    while (nb < 64 && (int64_t)nb * 2 * len <= 2048 && nb * 2 <= rows + 1 && per_row_bytes * nb * 2 <= cap)
        nb *= 2;
    return nb;
}

// Output rows per CTA of the spectral tap sum (a power of two up to 8;
// NDCONV_MAC_ROWS overrides): the rows of a CTA share their kernel row
// spectra and, where the register window applies, their data rows.  Taken
// only while the CTA's shared memory leaves room for two CTAs per SM
// (kMacSmem): measured on 2560-point rows, two rows per CTA (two CTAs per
// SM) ran 12 % faster than one, four rows (one CTA per SM) 15 % slower.
constexpr size_t kMacSmem = 110 * 1024;
constexpr int64_t kFillCtas = 2 * 152;  // two CTAs per SM of a GB300
int mac_rows_target() {
    static int v = 0;
    if (!v) {
        const char *e = getenv("NDCONV_MAC_ROWS");
        int r = (e && atoi(e) > 0) ? atoi(e) : 8;
        v = 1;
        while (v * 2 <= r && v < 8) v *= 2;
    }
    return v;
}

// Threads per row-pass CTA.  A launch of few CTAs is latency-bound: one
// butterfly of the stage with the most butterflies per thread in a single
// round where that fits 128..384 threads (e.g. 256 for a 2560-point
// transform of radices 16, 16, 10).  A launch of many CTAs is
// throughput-bound: 256, which keeps more CTAs resident, or 512 when shared
// memory leaves room for at most two CTAs per SM.
template <typename T> int row_threads(const RowArgs<T> &A, int64_t ctas, size_t sm) {
    if (ctas > kFewCtas) {
        const int t = ndconv_tune(NDCONV_TUNE_ROW_THREADS);  // the autotuner's choice
        if (t >= 32 && t <= 512 && t % 32 == 0 && t % A.nb == 0) return t;
        return sm > kSmemPerSm / 3 ? 512 : kThreads;
    }
    int maxw = 0;
    for (int i = 0; i < A.pl.nst; i++) maxw = std::max(maxw, (A.pl.L / A.pl.rad[i]) << A.lognb);
    if (maxw < 128 || maxw > kFewThreads) return kThreads;
    return (maxw + 31) / 32 * 32;
}

// n_inst instances (grid.y); A.spec_is etc. describe their spacing
template <typename T, int MODE> int launch_row_mode(const RowArgs<T> &A, size_t sm, unsigned grid, int n_inst,
                                                    cudaStream_t st) {
    const int64_t ctas = (int64_t)grid * n_inst;
    const int threads = row_threads(A, ctas, sm);
    if constexpr (std::is_same<T, float>::value) {
        if (ctas <= kFewCtas) {
            int st1 = ensure_smem(row_kernel<T, MODE, kFewThreads>);
            if (st1) return st1;
            row_kernel<T, MODE, kFewThreads><<<dim3(grid, (unsigned)n_inst), threads, sm, st>>>(A);
            ndconv_count_launch();
            NDCONV_CUDA_OK(cudaGetLastError());
            return NDCONV_OK;
        }
    }
    int st_ = ensure_smem(row_kernel<T, MODE, 512>);
    if (st_) return st_;
    row_kernel<T, MODE, 512><<<dim3(grid, (unsigned)n_inst), threads, sm, st>>>(A);
    ndconv_count_launch();
    NDCONV_CUDA_OK(cudaGetLastError());
    return NDCONV_OK;
}

// Fill nb / lognb and the launch shape of a row pass over n_inst instances.
// cap bounds the shared memory the rows per CTA may take (the persistent
// batch kernel has less than a launch of its own).  ROW_INV_MAC groups its
// output rows: CTA = (axis-0 index and segment, residue class c of o1 mod
// mac_g, group), rows o1 = c + mac_g (group nb + b); mac_g = d1 / s1 when
// s1 divides d1 (the rows then share a window of data rows), else 1.
template <typename T>
int prep_row(RowArgs<T> &A, int n_inst, int64_t &grid, size_t &sm, size_t cap = kFftSmemMax, bool fill = true) {
    using C = typename RowArgs<T>::C;
    const size_t per_row = sizeof(C) * 2 * padded_slots<C>(A.pl.L + 1) + sizeof(RowInfo);
    int64_t rows = A.n_rows;
    if (A.mode == ROW_INV_MAC) {
        const AxisGeom &a1 = A.g.ax[1];
        A.mac_win = (a1.d % a1.s) == 0;
        A.mac_g = A.mac_win ? (int)(a1.d / a1.s) : 1;
        if (A.mac_g > A.n1) A.mac_g = (int)A.n1;  // residue classes beyond the rows are empty
        if (A.mac_g < 1) A.mac_g = 1;
        rows = (A.n1 + A.mac_g - 1) / A.mac_g;  // rows of the largest residue class
    }
    A.nb = pick_nb(A.pl.L, rows, per_row, std::min(cap, kFftSmemMax));
    if (A.mode == ROW_INV_MAC) {
        if (const int t = ndconv_tune(NDCONV_TUNE_MAC_ROWS)) {
            // the autotuner's rows per CTA, as far as rows and shared memory allow
            A.nb = 1;
            while (A.nb < t && A.nb * 2 <= rows + 1 && per_row * A.nb * 2 <= std::min(cap, kFftSmemMax)) A.nb *= 2;
        } else {
            while (A.nb < mac_rows_target() && A.nb * 2 <= rows + 1 && per_row * A.nb * 2 <= std::min(cap, kMacSmem))
                A.nb *= 2;
            // a launch of its own should still give every SM two CTAs: fewer
            // rows per CTA for small problems (timed over 3,000 random
            // problems: one row per CTA is 1.06x the best grouping in the
            // geometric mean, the shared-kernel-row grouping 1.25x, while
            // large problems want the grouping)
            const int64_t sn = A.seg_n > 1 ? A.seg_n : 1;
            const int64_t outer = A.n_rows / (A.n1 * sn);
            while (fill && A.nb > 1 && outer * sn * A.mac_g * ((rows + A.nb - 1) / A.nb) * n_inst < kFillCtas)
                A.nb /= 2;
        }
        A.mac_gc = (rows + A.nb - 1) / A.nb;
    }
    A.lognb = ilog2(A.nb);
    sm = row_smem(A);
    if (sm > kFftSmemMax) return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "FFT row length exceeds shared memory");
    if (((int64_t)(A.pl.L + 1) << A.lognb) >= (int64_t)1 << 29)
        return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "FFT row too long");
    if (A.mode == ROW_INV_MAC) {
        const int64_t sn = A.seg_n > 1 ? A.seg_n : 1;
        const int64_t outer = A.n_rows / (A.n1 * sn);
        grid = outer * sn * A.mac_g * A.mac_gc;
    } else {
        grid = (A.n_rows + A.nb - 1) / A.nb;
    }
    if (grid > 0x7fffffff || n_inst > 65535) return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "too many FFT rows");
    return NDCONV_OK;
}

// n_inst instances (grid.y); A.spec_is etc. describe their spacing
template <typename T> int launch_row(RowArgs<T> A, cudaStream_t st, int n_inst = 1) {
    if (A.n_rows <= 0 || n_inst <= 0) return NDCONV_OK;
    int64_t grid;
    size_t sm;
    int s = prep_row(A, n_inst, grid, sm);
    if (s) return s;
    switch (A.mode) {
    case ROW_FWD_DATA: return launch_row_mode<T, ROW_FWD_DATA>(A, sm, (unsigned)grid, n_inst, st);
    case ROW_FWD_KERNEL: return launch_row_mode<T, ROW_FWD_KERNEL>(A, sm, (unsigned)grid, n_inst, st);
    case ROW_INV_OUT: return launch_row_mode<T, ROW_INV_OUT>(A, sm, (unsigned)grid, n_inst, st);
    case ROW_FUSED: return launch_row_mode<T, ROW_FUSED>(A, sm, (unsigned)grid, n_inst, st);
    case ROW_FWD_PLAIN: return launch_row_mode<T, ROW_FWD_PLAIN>(A, sm, (unsigned)grid, n_inst, st);
    case ROW_INV_MAC: return launch_row_mode<T, ROW_INV_MAC>(A, sm, (unsigned)grid, n_inst, st);
    default: return launch_row_mode<T, ROW_INV_PLAIN>(A, sm, (unsigned)grid, n_inst, st);
    }
}

// Two independent forward row passes in one launch (the kernel rows and the
// data rows of the row-spectral form): CTAs [0, ga) take pass A, the rest B.
template <typename T, int MAXT>
__global__ void __launch_bounds__(MAXT, 2) row_pair_kernel(const __grid_constant__ RowArgs<T> A,
                                                            const __grid_constant__ RowArgs<T> B, unsigned ga) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    if (blockIdx.x < ga) {
        if (fixed_rows(A) == 1) row_block<T, ROW_FWD_KERNEL, 2560, 1>(A, blockIdx.x, blockIdx.y, smem_raw);
        else row_block<T, ROW_FWD_KERNEL>(A, blockIdx.x, blockIdx.y, smem_raw);
    } else {
        if (fixed_rows(B) == 1) row_block<T, ROW_FWD_DATA, 2560, 1>(B, blockIdx.x - ga, blockIdx.y, smem_raw);
        else row_block<T, ROW_FWD_DATA>(B, blockIdx.x - ga, blockIdx.y, smem_raw);
    }
}

template <typename T> int launch_row_pair(RowArgs<T> A, RowArgs<T> B, cudaStream_t st, int n_inst) {
    if (n_inst <= 0) return NDCONV_OK;
    if (A.n_rows <= 0) return launch_row<T>(B, st, n_inst);
    if (B.n_rows <= 0) return launch_row<T>(A, st, n_inst);
    int64_t ga, gb;
    size_t sa, sb;
    int s = prep_row(A, n_inst, ga, sa);
    if (s) return s;
    if ((s = prep_row(B, n_inst, gb, sb))) return s;
    if (ga + gb > 0x7fffffff) return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "too many FFT rows");
    const int64_t ctas = (ga + gb) * n_inst;
    const int threads = std::max(row_threads(A, ctas, std::max(sa, sb)), row_threads(B, ctas, std::max(sa, sb)));
    const dim3 grid((unsigned)(ga + gb), (unsigned)n_inst);
    bool done = false;
    if constexpr (std::is_same<T, float>::value) {
        if (ctas <= kFewCtas) {
            if ((s = ensure_smem(row_pair_kernel<T, kFewThreads>))) return s;
            row_pair_kernel<T, kFewThreads><<<grid, threads, std::max(sa, sb), st>>>(A, B, (unsigned)ga);
            done = true;
        }
    }
    if (!done) {
        if ((s = ensure_smem(row_pair_kernel<T, 512>))) return s;
        row_pair_kernel<T, 512><<<grid, threads, std::max(sa, sb), st>>>(A, B, (unsigned)ga);
    }
    ndconv_count_launch();
    NDCONV_CUDA_OK(cudaGetLastError());
    return NDCONV_OK;
}

// Fill nb / lognb and the launch shape of a column pass.
template <typename C> int prep_col(ColArgs<C> &A, int64_t &gx, int64_t &gy, size_t &sm) {
    const int64_t F = A.pl.L;
    int nb = 1;
    while (nb < 32 && (int64_t)nb * 2 <= A.n_inner + 1 && sizeof(C) * 2 * F * nb * 2 <= 96 * 1024) nb *= 2;
    A.nb = nb;
    A.lognb = ilog2(nb);
    sm = sizeof(C) * 2 * padded_slots<C>(F * nb);
    if (sm > kFftSmemMax) return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "FFT column length exceeds shared memory");
    gx = (A.n_inner + nb - 1) / nb;
    gy = A.n_outer < 65535 ? A.n_outer : 65535;
    if (gx > 0x7fffffff) return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "too many FFT columns");
    return NDCONV_OK;
}

template <typename C> int launch_col(ColArgs<C> A, cudaStream_t st, int n_inst = 1) {
    if (A.n_outer <= 0 || A.n_inner <= 0 || n_inst <= 0) return NDCONV_OK;
    int64_t gx, gy;
    size_t sm;
    int s = prep_col(A, gx, gy, sm);
    if (s) return s;
    if (n_inst > 65535) return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "too many FFT instances");
    int st_ = ensure_smem(col_kernel<C>);
    if (st_) return st_;
    col_kernel<C><<<dim3((unsigned)gx, (unsigned)gy, (unsigned)n_inst), kThreads, sm, st>>>(A);
    ndconv_count_launch();
    NDCONV_CUDA_OK(cudaGetLastError());
    return NDCONV_OK;
}

template <typename C> int plan_with_tw(int64_t L, FftPlanDev &pl, const C **tw) {
    if (L > (1 << 24) || !make_plan((int)L, pl))
        return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "FFT length has a prime factor above 64");
    const C *st = nullptr;
    int s = get_twiddles<C>((int)L, &st, 1, &pl);
    if (s) return s;
    pl.tws = st;
    return get_twiddles<C>((int)L, tw);
}

// Row plans for a row of F samples: kind, transform plan + tables.
template <typename T> int row_plan(int64_t F, bool real, RowArgs<T> &A) {
    using C = typename RowArgs<T>::C;
    A.F = F;
    if (!real) {
        A.kind = RK_COMPLEX;
        A.H = F;
        A.twF = nullptr;
        return plan_with_tw<C>(F, A.pl, &A.tw);
    }
    if (F % 2 == 0) {
        A.kind = RK_REAL_EVEN;
        A.H = F / 2 + 1;
        int s = plan_with_tw<C>(F / 2, A.pl, &A.tw);
        if (s) return s;
        return get_twiddles<C>((int)F, &A.twF);
    }
    A.kind = RK_REAL_ODD;
    A.H = F / 2 + 1;
    A.twF = nullptr;
    return plan_with_tw<C>(F, A.pl, &A.tw);
}

// workspace: processor-owned (grow only) or stream-ordered per call
struct Workspace {
    ndconv_fft_processor *proc;
    cudaStream_t st;
    void *ptr = nullptr;
    bool owned = false;
    int get(size_t bytes, void **out);
    ~Workspace() {
        if (owned && ptr) cudaFreeAsync(ptr, st);
    }
};
}  // namespace

}  // namespace ndconv

struct ndconv_fft_processor {
    int32_t dtype;
    int64_t rp_origin_len;
    void *ws;
    size_t ws_bytes;
    int device;
    // baked kernel spectrum (ndconv_fft_processor_bake): valid for calls
    // whose geometry key and kernel pointer match
    void *kbuf = nullptr;
    size_t kbuf_bytes = 0;
    const void *kptr = nullptr;
    std::vector<unsigned char> kkey;
};

namespace ndconv {
namespace {
int Workspace::get(size_t bytes, void **out) {
    if (bytes == 0) bytes = 16;
    if (proc) {
        if (proc->ws_bytes < bytes) {
            if (proc->ws) {
                NDCONV_CUDA_OK(cudaStreamSynchronize(st));
                cudaFree(proc->ws);
                proc->ws = nullptr;
                proc->ws_bytes = 0;
            }
            NDCONV_CUDA_OK(cudaMalloc(&proc->ws, bytes));
            proc->ws_bytes = bytes;
        }
        *out = proc->ws;
        return NDCONV_OK;
    }
    NDCONV_CUDA_OK(cudaMallocAsync(&ptr, bytes, st));
    owned = true;
    *out = ptr;
    return NDCONV_OK;
}
}  // namespace

// ------------------------------------------------------------ conv_fft --
namespace {
// Shared plan of one conv_fft geometry.
template <typename T> struct FftConvPlan {
    using R = typename Elem<T>::Real;
    using C = typename CplxT<R>::type;
    int64_t P[3], F[3], H;
    int astar;
    int rs;  // row-spectral form: FFT along the contiguous axis only
    int64_t seg_n, seg_len;  // overlap-save segments of the contiguous axis (seg_n 1: whole rows)
    RowArgs<T> rk;  // row plan (kind, pl, tw, twF, F, H)
    FftPlanDev pl0, pl1;
    const C *tw0, *tw1;
    size_t nK, nS;  // complex elements of Kh and S per instance
};

// Row-spectral form vs full N-d FFT.  The row-spectral form skips the
// column transforms and their spectrum round trips (two launches instead of
// up to six) at the price of |K0 x K1| complex MACs per output bin, whose
// kernel spectra stop fitting in L2 as the leading kernel axes grow.  The
// choice is a linear model of log2(t_rs / t_nd) in log2 sizes, least-squares
// fitted to the measured times of both forms over 8,852 random f32 problems
// (2-D and 3-D, kernels up to 127 per axis); its picks cost 1.7 % over the
// faster form's total, where a flop model cost 2.7x.
template <typename T> bool rs_preferred(const Geom3<T> &g, const FftConvPlan<T> &cp) {
    const AxisGeom &A0 = g.ax[0], &A1 = g.ax[1];
    auto l = [](double v) { return v > 1 ? std::log2(v) : 0.0; };
    const double z = -3.1795 + 0.6571 * l((double)A0.K * A1.K) - 0.0275 * l((double)A0.out * A1.out) +
                     0.0556 * l((double)cp.H) - 0.5778 * l((double)cp.P[0] * cp.P[1]) +
                     0.5565 * l((double)cp.F[0] * cp.F[1]) - 0.1077 * l((double)A0.keff * A1.keff);
    return z < 0;
}

// A row pass holds a row of F samples in shared memory with one row per CTA?
template <typename T> bool row_len_fits(int64_t F) {
    using C = typename CplxT<typename Elem<T>::Real>::type;
    const bool even_real = !Elem<T>::kComplex && F % 2 == 0;
    const int64_t M = even_real ? F / 2 : F;
    if (M >= (1 << 28)) return false;
    const size_t bytes = ((sizeof(RowInfo) + 15) / 16) * 16 + sizeof(C) * 2 * padded_slots<C>(even_real ? M + 1 : M);
    return bytes <= kFftSmemMax;
}

// Overlap-save segments for a contiguous axis too long for one row pass:
// the transform length F (7-smooth, or a power of two) that minimises the
// modelled cost of all segments, seg_len = F - keff + 1 new outputs per
// segment.  False when even the longest row that fits holds no output
// beyond the kernel's extent.
template <typename T> bool seg_plan(const AxisGeom &a2, bool pow2, int64_t &F, int64_t &nseg, int64_t &len) {
    const bool real = !Elem<T>::kComplex;
    const int64_t need = (a2.out - 1) * a2.s + 1;  // padded positions from keff - 1 that outputs read
    static const int odd[] = {1, 3, 5, 7, 9, 15, 21, 25, 27, 35, 45, 49, 63, 75, 81, 105};
    double best = -1;
    for (int c : odd) {
        if (pow2 && c != 1) break;
        for (int64_t f = (int64_t)c * 2; f <= (int64_t)1 << 26; f *= 2) {
            if (f <= a2.keff) continue;
            if (!row_len_fits<T>(f)) break;
            FftPlanDev pl;
            const int64_t L = real ? f / 2 : f;
            if (!make_plan((int)L, pl)) continue;
            double stages = 0;
            for (int q = 0; q < pl.nst; q++) stages += stage_cost(pl.rad[q]);
            const int64_t l = f - a2.keff + 1;
            const int64_t n = (need + l - 1) / l;
            // forward + inverse transform, plus loads, stores and the spectral product
            double c_seg = 2.0 * (double)L * stages + 3.0 * (double)f;
            if (f > 8192) c_seg *= 1.15;  // fewer CTAs resident per SM
            const double cost = (double)n * c_seg;
            if (best < 0 || cost < best) {
                best = cost;
                F = f;
                nseg = n;
                len = l;
            }
        }
    }
    return best >= 0;
}

template <typename T> int make_conv_plan(const Geom3<T> &g, FftConvPlan<T> &cp, int variant = FFTV_AUTO) {
    using C = typename FftConvPlan<T>::C;
    const bool real = !Elem<T>::kComplex;
    const bool pow2 = (variant == FFTV_ND_POW2 || variant == FFTV_RS_POW2);
    for (int a = 0; a < 3; a++) {
        cp.P[a] = g.ax[a].L;
        cp.F[a] = (cp.P[a] == 1) ? 1 : (pow2 ? pow2_size(cp.P[a], real && a == 2) : smooth_size(cp.P[a], real && a == 2));
    }
    cp.astar = cp.F[0] > 1 ? 0 : (cp.F[1] > 1 ? 1 : 2);
    // row positions and output indices of the row kernels are 32-bit
    if (cp.P[2] >= ((int64_t)1 << 31) - 1) return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "FFT row longer than 2^31 samples");
    cp.seg_n = 1;
    cp.seg_len = 0;
    if (!row_len_fits<T>(cp.F[2])) {
        // rows too long for one CTA: overlap-save segments, row-spectral form
        if (variant == FFTV_ND || variant == FFTV_ND_POW2)
            return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "FFT row length exceeds shared memory");
        if (!seg_plan<T>(g.ax[2], pow2, cp.F[2], cp.seg_n, cp.seg_len))
            return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "FFT kernel row too long for overlap-save segments");
    }
    cp.rk = RowArgs<T>{};
    int s = row_plan<T>(cp.F[2], real, cp.rk);
    if (s) return s;
    cp.H = cp.rk.H;
    cp.nK = (size_t)cp.F[0] * cp.F[1] * cp.H;
    cp.nS = (cp.astar == 2) ? 0 : (size_t)cp.P[0] * cp.F[1] * cp.H;
    cp.rs = 0;
    // (leading axes too long for one column pass: the N-d form reports it and
    // conv_fft runs the direct kernels, which skip the taps that read only
    // padding; the row-spectral form would sum every one of them per bin)
    const bool want_rs = (variant == FFTV_RS || variant == FFTV_RS_POW2) || cp.seg_n > 1 ||
                         (variant == FFTV_AUTO && rs_preferred(g, cp));
    if (cp.astar < 2 && want_rs) {
        cp.rs = 1;
        const int64_t Hp = (cp.H + 1) & ~(int64_t)1;  // even row pitch (bin pairs as one vector)
        cp.nK = (size_t)g.ax[0].K * g.ax[1].K * Hp;
        cp.nS = (size_t)cp.P[0] * cp.P[1] * cp.seg_n * Hp;
    }
    cp.pl0 = FftPlanDev{};
    cp.pl1 = FftPlanDev{};
    cp.tw0 = cp.tw1 = nullptr;
    if (!cp.rs) {
        if (cp.F[0] > 1 && (s = plan_with_tw<C>(cp.F[0], cp.pl0, &cp.tw0))) return s;
        if (cp.F[1] > 1 && (s = plan_with_tw<C>(cp.F[1], cp.pl1, &cp.tw1))) return s;
    }
    return NDCONV_OK;
}

// Which passes conv_fft_passes emits: all, only the kernel spectrum, or
// only the data passes (kernel spectrum already in Kh).
enum : int { PASSES_ALL = 0, PASSES_KERNEL = 1, PASSES_DATA = 2 };

// The passes of instances [base, base + cnt), in order, handed to emit_row /
// emit_col (launch them, or record them as tasks).  Kh / S hold cnt
// instances' spectra back to back.  Pointers come from the device arrays
// xs / ks / ys when given, else x / k / y (cnt == 1).
template <typename T, typename EmitRow, typename EmitCol, typename EmitPair>
int conv_fft_passes(const Geom3<T> &g, int reverse, const FftConvPlan<T> &cp, const T *x, const T *k, T *y,
                    const T *const *xs, const T *const *ks, T *const *ys, int64_t base, int cnt,
                    typename FftConvPlan<T>::C *Kh, typename FftConvPlan<T>::C *S, EmitRow &&emit_row,
                    EmitCol &&emit_col, EmitPair &&emit_pair, int which = PASSES_ALL) {
    using R = typename Elem<T>::Real;
    using C = typename FftConvPlan<T>::C;
    const AxisGeom &A0 = g.ax[0], &A1 = g.ax[1], &A2 = g.ax[2];
    const int64_t *P = cp.P, *F = cp.F, H = cp.H;
    const int64_t K_is = (int64_t)cp.nK, S_is = (int64_t)cp.nS;
    int s;

    if (cp.rs) {
        const int64_t Hp = (H + 1) & ~(int64_t)1;  // row pitch of both spectra
        // ---- row-spectral form: kernel rows Kh[K0][K1][H] (tap order) and
        // padded data rows S[P0][P1][H] in one pass, then per output row the
        // sum over leading taps, inverse, crop
        RowArgs<T> kr = cp.rk;
        kr.mode = ROW_FWD_KERNEL;
        kr.kcompact = 1;
        kr.g = g;
        kr.k = k;
        kr.ks = ks;
        kr.inst_base = base;
        kr.reverse = reverse;
        kr.n1 = A1.K;
        kr.n_rows = A0.K * A1.K;
        kr.spec = Kh;
        kr.spec_s0 = A1.K * Hp;
        kr.spec_s1 = Hp;
        kr.spec_is = K_is;
        kr.scale = 1;
        // data spectra S[P0][P1][segment][H] (one segment unless the rows are long)
        const int64_t sn = cp.seg_n, Hs = sn * Hp;
        RowArgs<T> dr = cp.rk;
        dr.mode = ROW_FWD_DATA;
        dr.g = g;
        dr.x = x;
        dr.xs = xs;
        dr.inst_base = base;
        dr.n1 = P[1];
        dr.n_rows = P[0] * P[1] * sn;
        dr.seg_n = sn;
        dr.seg_len = cp.seg_len;
        dr.spec = S;
        dr.spec_s0 = P[1] * Hs;
        dr.spec_s1 = Hs;
        dr.spec_sg = Hp;
        dr.spec_is = S_is;
        dr.scale = 1;
        if (which == PASSES_KERNEL) return emit_row(kr, cnt);
        if ((s = (which == PASSES_DATA) ? emit_row(dr, cnt) : emit_pair(kr, dr, cnt))) return s;
        RowArgs<T> ir = cp.rk;
        ir.mode = ROW_INV_MAC;
        ir.g = g;
        ir.n1 = A1.out;
        ir.n_rows = A0.out * A1.out * sn;
        ir.seg_n = sn;
        ir.seg_len = cp.seg_len;
        ir.spec_sg = Hp;
        ir.spec = S;
        ir.spec_is = S_is;
        ir.kspec = Kh;
        ir.kspec_is = K_is;
        ir.mk0 = (int)A0.K;
        ir.mk1 = (int)A1.K;
        ir.mbase0 = A0.s * P[1] * Hs;
        ir.mbase1 = A1.s * Hs;
        ir.mstep0 = A0.d * P[1] * Hs;
        ir.mstep1 = A1.d * Hs;
        ir.mpitch = Hp;
        ir.y = y;
        ir.ys = ys;
        ir.inst_base = base;
        ir.y_s0 = A1.out * A2.out;
        ir.y_s1 = A2.out;
        ir.out_n = A2.out;
        ir.crop_off = A2.keff - 1;
        ir.crop_step = A2.s;
        ir.scale = (R)(1.0 / (double)F[2]);
        return emit_row(ir, cnt);
    }

    // ---- kernel spectrum
    RowArgs<T> kr = cp.rk;
    kr.mode = ROW_FWD_KERNEL;
    kr.g = g;
    kr.k = k;
    kr.ks = ks;
    kr.inst_base = base;
    kr.reverse = reverse;
    kr.n1 = A1.keff;
    kr.n_rows = A0.keff * A1.keff;
    kr.spec = Kh;
    kr.spec_s0 = F[1] * H;
    kr.spec_s1 = H;
    kr.spec_is = K_is;
    kr.scale = 1;
    if (which != PASSES_DATA && (s = emit_row(kr, cnt))) return s;
    if (F[1] > 1 && which != PASSES_DATA) {
        ColArgs<C> c{};
        c.mode = COL_FWD;
        c.src = c.dst = Kh;
        c.src_is = c.dst_is = K_is;
        c.n_inner = H;
        c.n_outer = A0.keff;
        c.src_outer = c.dst_outer = F[1] * H;
        c.src_axis = c.dst_axis = H;
        c.valid_in = A1.keff;
        c.pl = cp.pl1;
        c.tw = cp.tw1;
        if ((s = emit_col(c, cnt))) return s;
    }
    if (F[0] > 1 && which != PASSES_DATA) {
        ColArgs<C> c{};
        c.mode = COL_FWD;
        c.src = c.dst = Kh;
        c.src_is = c.dst_is = K_is;
        c.n_inner = F[1] * H;
        c.n_outer = 1;
        c.src_axis = c.dst_axis = F[1] * H;
        c.valid_in = A0.keff;
        c.pl = cp.pl0;
        c.tw = cp.tw0;
        if ((s = emit_col(c, cnt))) return s;
    }
    const R scale = (R)(1.0 / ((double)F[0] * (double)F[1] * (double)F[2]));
    if (which == PASSES_KERNEL) return NDCONV_OK;

    if (cp.astar == 2) {
        RowArgs<T> fr = cp.rk;
        fr.mode = ROW_FUSED;
        fr.g = g;
        fr.x = x;
        fr.xs = xs;
        fr.y = y;
        fr.ys = ys;
        fr.inst_base = base;
        fr.n1 = 1;
        fr.n_rows = cp.seg_n;
        fr.seg_n = cp.seg_n;
        fr.seg_len = cp.seg_len;
        fr.kspec = Kh;
        fr.kspec_is = K_is;
        fr.y_s0 = 0;
        fr.y_s1 = 0;
        fr.out_n = A2.out;
        fr.crop_off = A2.keff - 1;
        fr.crop_step = A2.s;
        fr.scale = scale;
        return emit_row(fr, cnt);
    }

    // ---- data: forward row pass into S
    RowArgs<T> dr = cp.rk;
    dr.mode = ROW_FWD_DATA;
    dr.g = g;
    dr.x = x;
    dr.xs = xs;
    dr.inst_base = base;
    dr.n1 = P[1];
    dr.n_rows = P[0] * P[1];
    dr.spec = S;
    dr.spec_s0 = F[1] * H;
    dr.spec_s1 = H;
    dr.spec_is = S_is;
    dr.scale = 1;
    if ((s = emit_row(dr, cnt))) return s;
    if (cp.astar == 0 && F[1] > 1) {
        ColArgs<C> c{};
        c.mode = COL_FWD;
        c.src = c.dst = S;
        c.src_is = c.dst_is = S_is;
        c.n_inner = H;
        c.n_outer = P[0];
        c.src_outer = c.dst_outer = F[1] * H;
        c.src_axis = c.dst_axis = H;
        c.valid_in = P[1];
        c.pl = cp.pl1;
        c.tw = cp.tw1;
        if ((s = emit_col(c, cnt))) return s;
    }
    {
        ColArgs<C> c{};
        c.mode = COL_FUSED;
        c.src = c.dst = S;
        c.src_is = c.dst_is = S_is;
        c.n_outer = 1;
        c.kspec = Kh;
        c.k_is = K_is;
        if (cp.astar == 0) {
            c.n_inner = F[1] * H;
            c.src_axis = c.dst_axis = F[1] * H;
            c.valid_in = P[0];
            c.k_axis = F[1] * H;
            c.crop_off = A0.keff - 1;
            c.crop_step = A0.s;
            c.n_out = A0.out;
            c.pl = cp.pl0;
            c.tw = cp.tw0;
        } else {
            c.n_inner = H;
            c.src_axis = c.dst_axis = H;
            c.valid_in = P[1];
            c.k_axis = H;
            c.crop_off = A1.keff - 1;
            c.crop_step = A1.s;
            c.n_out = A1.out;
            c.pl = cp.pl1;
            c.tw = cp.tw1;
        }
        if ((s = emit_col(c, cnt))) return s;
    }
    if (cp.astar == 0 && F[1] > 1) {
        ColArgs<C> c{};
        c.mode = COL_INV;
        c.src = c.dst = S;
        c.src_is = c.dst_is = S_is;
        c.n_inner = H;
        c.n_outer = A0.out;
        c.src_outer = c.dst_outer = F[1] * H;
        c.src_axis = c.dst_axis = H;
        c.valid_in = F[1];
        c.crop_off = A1.keff - 1;
        c.crop_step = A1.s;
        c.n_out = A1.out;
        c.pl = cp.pl1;
        c.tw = cp.tw1;
        if ((s = emit_col(c, cnt))) return s;
    }
    RowArgs<T> ir = cp.rk;
    ir.mode = ROW_INV_OUT;
    ir.n1 = A1.out;
    ir.n_rows = A0.out * A1.out;
    ir.spec = S;
    ir.spec_s0 = F[1] * H;
    ir.spec_s1 = H;
    ir.spec_is = S_is;
    ir.y = y;
    ir.ys = ys;
    ir.inst_base = base;
    ir.y_s0 = A1.out * A2.out;
    ir.y_s1 = A2.out;
    ir.out_n = A2.out;
    ir.crop_off = A2.keff - 1;
    ir.crop_step = A2.s;
    ir.scale = scale;
    return emit_row(ir, cnt);
}

template <typename T>
int conv_fft_wave(const Geom3<T> &g, int reverse, const FftConvPlan<T> &cp, const T *x, const T *k, T *y,
                  const T *const *xs, const T *const *ks, T *const *ys, int64_t base, int cnt,
                  typename FftConvPlan<T>::C *Kh, typename FftConvPlan<T>::C *S, cudaStream_t st,
                  int which = PASSES_ALL) {
    using C = typename FftConvPlan<T>::C;
    return conv_fft_passes<T>(
        g, reverse, cp, x, k, y, xs, ks, ys, base, cnt, Kh, S,
        [&](RowArgs<T> &A, int n) { return launch_row<T>(A, st, n); },
        [&](ColArgs<C> &A, int n) { return launch_col<C>(A, st, n); },
        [&](RowArgs<T> &A, RowArgs<T> &B, int n) { return launch_row_pair<T>(A, B, st, n); }, which);
}

// bytes of spectra a wave may keep so that they stay in L2 between passes
// Spectra bytes one wave of a batch may hold.  Large waves win: the two
// launches of a wave fill the GPU with many CTAs (short tails), and the
// spectra that spill from L2 cost little next to the transforms (measured
// on the 2-D case: 387 / 398 / 436 / 465 GB/s at 24 / 48 / 128 / 512 MB).
// Capped by a quarter of the device memory free at first use.
size_t wave_budget_bytes() {
    static size_t v = 0;
    if (!v) {
        const char *e = getenv("NDCONV_WAVE_MB");
        v = (size_t)((e && atoi(e) > 0) ? atoi(e) : 1024) << 20;
        size_t fr = 0, tot = 0;
        if (!(e && atoi(e) > 0) && cudaMemGetInfo(&fr, &tot) == cudaSuccess && fr / 4 < v) v = fr / 4;
        if (v < ((size_t)16 << 20)) v = (size_t)16 << 20;
    }
    return v;
}
}  // namespace
}  // namespace ndconv
