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
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "fft.h"
#include "fft_core.cuh"

namespace ndconv {

// ------------------------------------------------------------- twiddles --
template <typename C>
__global__ void gen_twiddles_kernel(C *tw, int L) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < L; t += gridDim.x * blockDim.x) {
        double s, c;
        sincospi(-2.0 * (double)t / (double)L, &s, &c);  // exp(-2 pi i t / L) in FP64
        tw[t].re = (decltype(tw[t].re))c;
        tw[t].im = (decltype(tw[t].im))s;
    }
}

thread_local TwArena *g_tw_arena = nullptr;

TwArenaScope::TwArenaScope(TwArena *a) : prev(g_tw_arena) { g_tw_arena = a; }
TwArenaScope::~TwArenaScope() { g_tw_arena = prev; }

namespace {
std::mutex g_tw_mu;
std::map<std::tuple<int, int, int>, void *> g_tw;  // (device, bytes-per-complex, L) -> table

// Tables carved from a caller-provided arena and generated on its stream
// (no allocation, no synchronisation).
template <typename C> int arena_twiddles(TwArena *a, int L, const C **out) {
    for (int i = 0; i < a->n; i++)
        if (a->len[i] == L && a->elem[i] == (int)sizeof(C)) {
            *out = (const C *)a->table[i];
            return NDCONV_OK;
        }
    const size_t off = (a->used + 255) / 256 * 256;
    const size_t bytes = sizeof(C) * (size_t)(L > 0 ? L : 1);
    if (a->n >= TwArena::kMaxTables || off + bytes > a->cap)
        return ndconv_fail(NDCONV_ERR_NO_MEMORY, "twiddle tables do not fit the provided scratch");
    C *p = reinterpret_cast<C *>(a->base + off);
    int blocks = (L + 255) / 256;
    if (blocks > 1024) blocks = 1024;
    if (blocks < 1) blocks = 1;
    gen_twiddles_kernel<C><<<blocks, 256, 0, a->st>>>(p, L);
    ndconv_count_launch();
    NDCONV_CUDA_OK(cudaGetLastError());
    a->used = off + bytes;
    a->len[a->n] = L;
    a->elem[a->n] = (int)sizeof(C);
    a->table[a->n] = p;
    a->n++;
    *out = p;
    return NDCONV_OK;
}

template <typename C> int get_twiddles(int L, const C **out) {
    if (g_tw_arena) return arena_twiddles<C>(g_tw_arena, L, out);
    int dev = 0;
    NDCONV_CUDA_OK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_tw_mu);
    auto key = std::make_tuple(dev, (int)sizeof(C), L);
    auto it = g_tw.find(key);
    if (it != g_tw.end()) {
        *out = (const C *)it->second;
        return NDCONV_OK;
    }
    void *p = nullptr;
    NDCONV_CUDA_OK(cudaMalloc(&p, sizeof(C) * (size_t)(L > 0 ? L : 1)));
    cudaStream_t s;
    NDCONV_CUDA_OK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    int blocks = (L + 255) / 256;
    if (blocks > 1024) blocks = 1024;
    if (blocks < 1) blocks = 1;
    gen_twiddles_kernel<C><<<blocks, 256, 0, s>>>((C *)p, L);
    ndconv_count_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (e != cudaSuccess) {
        cudaFree(p);
        return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
    }
    g_tw[key] = p;
    *out = (const C *)p;
    return NDCONV_OK;
}
}  // namespace

// Radix factorisation: 8s, 4, 2, 3s, 5s, then other primes (generic
// butterfly up to kMaxGenericRadix).  Returns false if a prime factor is
// larger than that.
// Radices: 16s for the power of two (one radix-10 stage takes a factor 2
// with a factor 5, then 8 / 4 / 2 for the rest), then odd factors.  Fewer,
// wider stages mean fewer shared-memory round trips and barriers.
bool make_plan(int L, FftPlanDev &pl) {
    pl.L = L;
    pl.nst = 0;
    int r = L;
    const bool ten = (r % 10 == 0) && (r % 4 != 0 || r % 32 == 0);
    if (ten) r /= 10;
    while (r % 16 == 0) { pl.rad[pl.nst++] = 16; r /= 16; }
    if (r % 8 == 0) { pl.rad[pl.nst++] = 8; r /= 8; }
    if (r % 4 == 0) { pl.rad[pl.nst++] = 4; r /= 4; }
    if (r % 2 == 0) { pl.rad[pl.nst++] = 2; r /= 2; }
    if (ten) pl.rad[pl.nst++] = 10;
    for (int f = 3; r > 1; f += 2) {
        while (r % f == 0) {
            if (f > kMaxGenericRadix || pl.nst >= kMaxStages) return false;
            pl.rad[pl.nst++] = f;
            r /= f;
        }
        if ((int64_t)f * f > r && r > 1) {
            if (r > kMaxGenericRadix || pl.nst >= kMaxStages) return false;
            pl.rad[pl.nst++] = r;
            r = 1;
        }
    }
    uint32_t ns = 1;
    for (int s = 0; s < pl.nst; s++) {
        pl.ns[s] = make_fastdiv(ns);
        ns *= (uint32_t)pl.rad[s];
    }
    return true;
}

// Relative cost of one Stockham stage per element, by radix (each stage is
// one shared-memory round trip; larger radices do more arithmetic).
static double stage_cost(int r) {
    switch (r) {
    case 16: return 1.25;
    case 10: return 1.2;
    case 8: return 1.0;
    case 4: return 0.75;
    case 2: return 0.6;
    case 3: return 0.8;
    case 5: return 1.0;
    case 7: return 1.3;
    default: return 4.0;
    }
}

// Cheapest 2^a 3^b 5^c 7^d >= n (even when asked; the real axis transforms
// half of it), among sizes up to 1.35 n.
int64_t smooth_size(int64_t n, bool even) {
    if (n <= 1) return even ? 2 : 1;
    int64_t best = INT64_MAX;
    double best_cost = 1e300;
    const int64_t lim = n + n * 35 / 100 + 8;
    for (int64_t p7 = 1; p7 <= 4 * lim; p7 *= 7)
        for (int64_t p5 = p7; p5 <= 4 * lim; p5 *= 5)
            for (int64_t p3 = p5; p3 <= 4 * lim; p3 *= 3) {
                int64_t v = p3;
                while (v < n || (even && (v & 1))) v *= 2;
                if (v > lim && best != INT64_MAX) continue;
                FftPlanDev pl;
                const int64_t L = even ? v / 2 : v;
                double c = 1e300;
                if (L < (1 << 30) && make_plan((int)L, pl)) {
                    c = 0;
                    for (int s = 0; s < pl.nst; s++) c += stage_cost(pl.rad[s]);
                    c *= (double)L;
                }
                if (c < best_cost || (c == best_cost && v < best)) {
                    best_cost = c;
                    best = v;
                }
            }
    return best;
}

int64_t pow2_size(int64_t n, bool even) {
    int64_t v = even ? 2 : 1;
    while (v < n) v *= 2;
    return v;
}

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
    int64_t mpitch;          // INV_MAC: row pitch of both spectra (even: bin pairs load as one vector)
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

// r2c post-processing: X[k] (k = 0..M) from Z = FFT_M(x[2m] + i x[2m+1])
template <typename C>
__device__ void r2c_post(const C *Z, C *X, int M, int nb, int lognb, const C *__restrict__ twF) {
    using R = decltype(Z[0].re);
    const int total = (M + 1) << lognb;
    for (int u = threadIdx.x; u < total; u += blockDim.x) {
        const int b = u & (nb - 1);
        const int k = u >> lognb;
        const C a = Z[sx<C>(((k == M ? 0 : k) << lognb) + b)];
        const C c = cconj(Z[sx<C>(((k == 0 ? 0 : M - k) << lognb) + b)]);
        const C e = C{(R)0.5 * (a.re + c.re), (R)0.5 * (a.im + c.im)};
        const C d = C{(R)0.5 * (a.re - c.re), (R)0.5 * (a.im - c.im)};
        const C o = C{d.im, -d.re};  // -i * d
        const C wo = cmul(twF[k], o);
        X[sx<C>(u)] = C{e.re + wo.re, e.im + wo.im};
    }
}

// c2r pre-processing: Z[k] (k < M) such that IFFT_M(Z)[j] = x[2j] + i x[2j+1]
// for the unnormalised length-2M inverse of the Hermitian spectrum X[0..M]
// (imaginary parts of the DC and Nyquist bins ignored).
template <typename C>
__device__ void c2r_pre(const C *X, C *Z, int M, int nb, int lognb, const C *__restrict__ twF) {
    const int total = M << lognb;
    for (int u = threadIdx.x; u < total; u += blockDim.x) {
        const int b = u & (nb - 1);
        const int k = u >> lognb;
        C a = X[sx<C>(u)], c = X[sx<C>(((M - k) << lognb) + b)];
        if (k == 0) {
            a.im = 0;
            c.im = 0;
        }
        c = cconj(c);
        const C e = cadd(a, c);
        const C d = csub(a, c);
        const C o = cmul(d, cconj(twF[k]));
        Z[sx<C>(u)] = C{e.re - o.im, e.im + o.re};  // e + i*o
    }
}

// One CTA's share of a row pass: rows [bx * nb, bx * nb + nb) of instance by.
template <typename T, int MODE>
__device__ __forceinline__ void row_block(const RowArgs<T> &A, unsigned bx, unsigned by, unsigned char *smem_raw) {
    using C = typename RowArgs<T>::C;
    using R = typename RowArgs<T>::R;
    const int nb = A.nb, lognb = A.lognb;
    const int M = A.pl.L;  // transform length
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

    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        const int64_t r = rbase + b;
        const int64_t sn = A.seg_n > 1 ? A.seg_n : 1;
        const int64_t rr = r / sn, seg = r - rr * sn;
        const int64_t i0 = rr / A.n1, i1 = rr - i0 * A.n1;
        RowInfo ri{};
        ri.valid = r < A.n_rows;
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
    C *res;
    if constexpr (fwd) {
        // ---- load samples: element (b, i) -> buf0[i * nb + b], four independent loads per round
        const int total = M << lognb;
        const int T_ = blockDim.x;
        for (int u0 = threadIdx.x; u0 < total; u0 += 4 * T_) {
            C v[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int u = u0 + q * T_;
                v[q] = C{0, 0};
                if (u < total) {
                    const int b = bt, i = u >> lognb;
                    const RowInfo &ri = rit;
                    if (ri.valid) {
                        const int64_t r = rbase + b;
                        if (A.kind == RK_REAL_EVEN) {
                            const T s0 = row_sample<MODE>(A, x, kp, ri, r, 2 * (int64_t)i);
                            const T s1 = row_sample<MODE>(A, x, kp, ri, r, 2 * (int64_t)i + 1);
                            v[q] = C{RealPart<T>::re(s0), RealPart<T>::re(s1)};
                        } else {
                            const T s = row_sample<MODE>(A, x, kp, ri, r, i);
                            v[q] = C{RealPart<T>::re(s), RealPart<T>::im(s)};
                        }
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int u = u0 + q * T_;
                if (u < total) buf0[sx<C>(u)] = v[q];
            }
        }
        __syncthreads();
        res = block_fft<false>(buf0, buf1, nb, lognb, A.pl, A.tw);
        C *other = (res == buf0) ? buf1 : buf0;
        if (A.kind == RK_REAL_EVEN) {
            r2c_post(res, other, M, nb, lognb, A.twF);
            __syncthreads();
            C *t = res;
            res = other;
            other = t;
        }
        const int H = (int)A.H;
        if constexpr (MODE != ROW_FUSED) {
            const int tot = H << lognb;
            if (rit.valid)
                for (int u = threadIdx.x; u < tot; u += blockDim.x) spec[rit.soff + (u >> lognb)] = res[sx<C>(u)];
            return;
        }
        // ---- fused: multiply by the kernel spectrum, back to the time domain
        {
            const int tot = H << lognb;
            for (int u = threadIdx.x; u < tot; u += blockDim.x) res[sx<C>(u)] = cmul(res[sx<C>(u)], ldcg_c(kspec + (u >> lognb)));
            __syncthreads();
        }
        if (A.kind == RK_REAL_EVEN) {
            c2r_pre(res, other, M, nb, lognb, A.twF);
            __syncthreads();
            res = block_fft<true>(other, res, nb, lognb, A.pl, A.tw);
        } else {
            res = block_fft<true>(res, other, nb, lognb, A.pl, A.tw);
        }
    } else {
        // ---- inverse: load spectrum rows
        const int H = (int)A.H;
        const int tot = H << lognb;
        C *dst = (A.kind == RK_REAL_EVEN) ? buf1 : buf0;
        if constexpr (MODE == ROW_INV_MAC) {
            // output row spectrum = sum over leading taps (tz, ty) of kernel row
            // (tz, ty) times data row (o0 s0 + tz d0, o1 s1 + ty d1); four bins
            // per thread at a time so that eight loads are in flight per tap
            const int mk0 = A.mk0, mk1 = A.mk1;
            const int64_t st0 = A.mstep0, st1 = A.mstep1, Hh = A.mpitch;
            const bool l2 = A.l2only;
            const int T_ = blockDim.x;
            bool vec_done = false;
            if constexpr (sizeof(C) == 8) {
                if (nb == 1 && (Hh & 1) == 0) {
                    // one row per CTA, even pitch: bins (2p, 2p + 1) as one 16-byte
                    // load of each spectrum (half the requests in flight for the same bytes)
                    const int npair = (H + 1) >> 1;
                    const float4 *kv4 = reinterpret_cast<const float4 *>(kspec);
                    const float4 *sv4 = reinterpret_cast<const float4 *>(spec + rit.soff);
                    for (int p0 = threadIdx.x; p0 < npair; p0 += 4 * T_) {
                        float4 acc[4];
                        int pq[4];
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            const int pp = p0 + q * T_;
                            pq[q] = (pp < npair && rit.valid) ? pp : 0;
                            acc[q] = make_float4(0.f, 0.f, 0.f, 0.f);
                        }
                        auto taps = [&](auto load) {
                            for (int tz = 0; tz < mk0; tz++) {
                                for (int ty = 0; ty < mk1; ty++) {
                                    const int64_t so = (tz * st0 + ty * st1) >> 1, ko = ((int64_t)(tz * mk1 + ty) * Hh) >> 1;
                                    float4 kv[4], dv[4];
#pragma unroll
                                    for (int q = 0; q < 4; q++) {
                                        kv[q] = load(kv4 + ko + pq[q]);
                                        dv[q] = load(sv4 + so + pq[q]);
                                    }
#pragma unroll
                                    for (int q = 0; q < 4; q++) {
                                        acc[q].x = fmaf(kv[q].x, dv[q].x, fmaf(-kv[q].y, dv[q].y, acc[q].x));
                                        acc[q].y = fmaf(kv[q].x, dv[q].y, fmaf(kv[q].y, dv[q].x, acc[q].y));
                                        acc[q].z = fmaf(kv[q].z, dv[q].z, fmaf(-kv[q].w, dv[q].w, acc[q].z));
                                        acc[q].w = fmaf(kv[q].z, dv[q].w, fmaf(kv[q].w, dv[q].z, acc[q].w));
                                    }
                                }
                            }
                        };
                        if (l2) taps([](const float4 *p) { return __ldcg(p); });
                        else taps([](const float4 *p) { return __ldg(p); });
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            const int pp = p0 + q * T_;
                            if (pp >= npair) continue;
                            const bool v = rit.valid;
                            dst[sx<C>(2 * pp)] = v ? C{acc[q].x, acc[q].y} : C{0, 0};
                            if (2 * pp + 1 < H) dst[sx<C>(2 * pp + 1)] = v ? C{acc[q].z, acc[q].w} : C{0, 0};
                        }
                    }
                    vec_done = true;
                }
            }
            for (int u0 = threadIdx.x; !vec_done && u0 < tot; u0 += 4 * T_) {
                C acc[4];
                int64_t soff[4], koff[4];
                bool ok[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int u = u0 + q * T_;
                    const int k = u >> lognb;
                    ok[q] = u < tot && rit.valid;
                    soff[q] = ok[q] ? rit.soff + k : 0;
                    koff[q] = ok[q] ? k : 0;
                    acc[q] = C{0, 0};
                }
                const C *kq[4], *sq[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    kq[q] = kspec + koff[q];
                    sq[q] = spec + soff[q];
                }
                auto taps = [&](auto load) {
                    for (int tz = 0; tz < mk0; tz++) {
                        for (int ty = 0; ty < mk1; ty++) {
                            const int64_t so = tz * st0 + ty * st1, ko = (int64_t)(tz * mk1 + ty) * Hh;
                            C kv[4], dv[4];
#pragma unroll
                            for (int q = 0; q < 4; q++) {
                                kv[q] = load(kq[q] + ko);
                                dv[q] = load(sq[q] + so);
                            }
#pragma unroll
                            for (int q = 0; q < 4; q++) {
                                acc[q].re = fmaf_t(kv[q].re, dv[q].re, fmaf_t(-kv[q].im, dv[q].im, acc[q].re));
                                acc[q].im = fmaf_t(kv[q].re, dv[q].im, fmaf_t(kv[q].im, dv[q].re, acc[q].im));
                            }
                        }
                    }
                };
                // the load kind is uniform: one loop nest per kind, no per-load select
                if (l2) taps([](const C *p) { return ldcg_c(p); });
                else taps([](const C *p) { return ldg_c(p); });
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int u = u0 + q * T_;
                    if (u < tot) dst[sx<C>(u)] = ok[q] ? acc[q] : C{0, 0};
                }
            }
        } else {
            for (int u = threadIdx.x; u < tot; u += blockDim.x)
                dst[sx<C>(u)] = rit.valid ? ldcg_c(spec + rit.soff + (u >> lognb)) : C{0, 0};
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
        if (A.kind == RK_REAL_EVEN) {
            c2r_pre(buf1, buf0, M, nb, lognb, A.twF);
            __syncthreads();
        }
        res = block_fft<true>(buf0, buf1, nb, lognb, A.pl, A.tw);
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
__global__ void __launch_bounds__(256) col_kernel(const __grid_constant__ ColArgs<C> A) {
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
int pick_nb(int64_t len, int64_t rows, size_t per_row_bytes) {
    int nb = 1;
    while (nb < 64 && (int64_t)nb * 2 * len <= 2048 && nb * 2 <= rows + 1 &&
           per_row_bytes * nb * 2 <= kFftSmemMax)
        nb *= 2;
    return nb;
}

// Threads per row-pass CTA.  A launch of few CTAs is latency-bound: one
// butterfly of the stage with the most butterflies per thread in a single
// round where that fits 128..384 threads (e.g. 256 for a 2560-point
// transform of radices 16, 16, 10).  A launch of many CTAs is
// throughput-bound: 256, which keeps more CTAs resident.
template <typename T> int row_threads(const RowArgs<T> &A, int64_t ctas) {
    if (ctas > kFewCtas) return kThreads;
    int maxw = 0;
    for (int i = 0; i < A.pl.nst; i++) maxw = std::max(maxw, (A.pl.L / A.pl.rad[i]) << A.lognb);
    if (maxw < 128 || maxw > kFewThreads) return kThreads;
    return (maxw + 31) / 32 * 32;
}

// n_inst instances (grid.y); A.spec_is etc. describe their spacing
template <typename T, int MODE> int launch_row_mode(const RowArgs<T> &A, size_t sm, unsigned grid, int n_inst,
                                                    cudaStream_t st) {
    const int64_t ctas = (int64_t)grid * n_inst;
    const int threads = row_threads(A, ctas);
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
template <typename T> int prep_row(RowArgs<T> &A, int n_inst, int64_t &grid, size_t &sm) {
    using C = typename RowArgs<T>::C;
    const size_t per_row = sizeof(C) * 2 * padded_slots<C>(A.pl.L + 1) + sizeof(RowInfo);
    A.nb = pick_nb(A.pl.L, A.n_rows, per_row);
    A.lognb = ilog2(A.nb);
    sm = row_smem(A);
    if (sm > kFftSmemMax) return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "FFT row length exceeds shared memory");
    if (((int64_t)(A.pl.L + 1) << A.lognb) >= (int64_t)1 << 29)
        return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "FFT row too long");
    grid = (A.n_rows + A.nb - 1) / A.nb;
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
    if (blockIdx.x < ga) row_block<T, ROW_FWD_KERNEL>(A, blockIdx.x, blockIdx.y, smem_raw);
    else row_block<T, ROW_FWD_DATA>(B, blockIdx.x - ga, blockIdx.y, smem_raw);
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
    const int threads = std::max(row_threads(A, ctas), row_threads(B, ctas));
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

// bytes that identify a geometry for a baked kernel spectrum
template <typename T> std::vector<unsigned char> bake_key(const Geom3<T> &g, int reverse) {
    std::vector<unsigned char> key(sizeof(Geom3<T>) + sizeof(int) + 1);
    Geom3<T> gz;
    memset(&gz, 0, sizeof(gz));
    for (int a = 0; a < 3; a++) {
        gz.ax[a] = g.ax[a];
        gz.ax[a].xs = 0;  // data strides do not change the kernel spectrum
        gz.cf[a] = g.cf[a];
        gz.cb[a] = g.cb[a];
    }
    memcpy(key.data(), &gz, sizeof(gz));
    memcpy(key.data() + sizeof(gz), &reverse, sizeof(int));
    key.back() = (unsigned char)sizeof(T);
    return key;
}

template <typename T>
int conv_fft_run(const Geom3<T> &g, int reverse, const T *x, const T *k, T *y,
                 ndconv_fft_processor *proc, cudaStream_t st, void *scratch, size_t scratch_bytes, int variant) {
    using C = typename FftConvPlan<T>::C;
    FftConvPlan<T> cp;
    int s = make_conv_plan(g, cp, variant);
    if (s) return s;
    const size_t bytes = sizeof(C) * (cp.nK + cp.nS) + 256;
    Workspace ws{proc, st};
    void *base = scratch;
    if (base) {
        if (scratch_bytes < bytes) return ndconv_fail(NDCONV_ERR_NO_MEMORY, "scratch too small");
    } else if ((s = ws.get(bytes, &base))) {
        return s;
    }
    C *Kh = reinterpret_cast<C *>(base);
    C *S = Kh + cp.nK;
    if (proc && proc->kbuf && proc->kptr == (const void *)k && variant == FFTV_AUTO &&
        proc->kkey == bake_key<T>(g, reverse))
        return conv_fft_wave<T>(g, reverse, cp, x, k, y, nullptr, nullptr, nullptr, 0, 1,
                                static_cast<C *>(proc->kbuf), S, st, PASSES_DATA);
    return conv_fft_wave<T>(g, reverse, cp, x, k, y, nullptr, nullptr, nullptr, 0, 1, Kh, S, st);
}

template <typename T>
int conv_fft_bake(const Geom3<T> &g, int reverse, const T *k, ndconv_fft_processor *proc, cudaStream_t st) {
    using C = typename FftConvPlan<T>::C;
    FftConvPlan<T> cp;
    int s = make_conv_plan(g, cp, FFTV_AUTO);
    if (s) return s;
    const size_t bytes = sizeof(C) * cp.nK + 256;
    if (proc->kbuf_bytes < bytes) {
        if (proc->kbuf) {
            NDCONV_CUDA_OK(cudaStreamSynchronize(st));
            cudaFree(proc->kbuf);
            proc->kbuf = nullptr;
            proc->kbuf_bytes = 0;
        }
        NDCONV_CUDA_OK(cudaMalloc(&proc->kbuf, bytes));
        proc->kbuf_bytes = bytes;
    }
    proc->kptr = nullptr;
    proc->kkey.clear();
    s = conv_fft_wave<T>(g, reverse, cp, nullptr, k, nullptr, nullptr, nullptr, nullptr, 0, 1,
                         static_cast<C *>(proc->kbuf), nullptr, st, PASSES_KERNEL);
    if (s) return s;
    proc->kptr = k;
    proc->kkey = bake_key<T>(g, reverse);
    return NDCONV_OK;
}

template <typename T>
int conv_fft_batch_run(const Geom3<T> &g, int reverse, int64_t n, const T *const *xs, const T *const *ks,
                       T *const *ys, ndconv_fft_processor *proc, cudaStream_t st, int variant) {
    using C = typename FftConvPlan<T>::C;
    if (n <= 0) return NDCONV_OK;
    FftConvPlan<T> cp;
    int s = make_conv_plan(g, cp, variant);
    if (s) return s;
    const size_t per = sizeof(C) * (cp.nK + cp.nS);
    int64_t W = (int64_t)(wave_budget_bytes() / (per ? per : 1));
    if (W < 1) W = 1;
    if (W > n) W = n;
    if (W > 65535) W = 65535;
    Workspace ws{proc, st};
    void *base = nullptr;
    if ((s = ws.get(per * W + 256, &base))) return s;
    C *Kh = reinterpret_cast<C *>(base);
    C *S = Kh + cp.nK * W;
    for (int64_t b = 0; b < n; b += W) {
        const int cnt = (int)(n - b < W ? n - b : W);
        if ((s = conv_fft_wave<T>(g, reverse, cp, nullptr, nullptr, nullptr, xs, ks, ys, b, cnt, Kh, S, st)))
            return s;
    }
    return NDCONV_OK;
}

// Spectra bytes of whichever FFT form needs more.
template <typename T> size_t conv_fft_scratch_bytes(const Geom3<T> &g, int variant) {
    using R = typename Elem<T>::Real;
    using C = typename CplxT<R>::type;
    const bool real = !Elem<T>::kComplex;
    const bool pow2 = (variant == FFTV_ND_POW2 || variant == FFTV_RS_POW2);
    int64_t P[3] = {g.ax[0].L, g.ax[1].L, g.ax[2].L}, F[3];
    for (int a = 0; a < 3; a++)
        F[a] = (P[a] == 1) ? 1 : (pow2 ? pow2_size(P[a], real && a == 2) : smooth_size(P[a], real && a == 2));
    const int astar = F[0] > 1 ? 0 : (F[1] > 1 ? 1 : 2);
    int64_t sn = 1, sl = 0;
    if (!row_len_fits<T>(F[2])) {
        if (!seg_plan<T>(g.ax[2], pow2, F[2], sn, sl)) return 256;  // unsupported: the plan reports it
    }
    const int64_t H = real ? F[2] / 2 + 1 : F[2];
    const size_t nK = (size_t)F[0] * F[1] * H;
    const size_t nS = (astar == 2) ? 0 : (size_t)P[0] * F[1] * H;
    // the row-spectral form: kernel rows and padded data rows (segments) (even row pitch)
    const size_t rs = (astar == 2) ? 0 : (size_t)(g.ax[0].K * g.ax[1].K + P[0] * P[1] * sn) * ((H + 1) & ~(int64_t)1);
    return sizeof(C) * std::max(sn > 1 ? nK : nK + nS, rs) + 256;
}

#define NDCONV_INST_FFT(T)                                                                          \
    template int conv_fft_run<T>(const Geom3<T> &, int, const T *, const T *, T *,                \
                                 ndconv_fft_processor *, cudaStream_t, void *, size_t, int);     \
    template int conv_fft_batch_run<T>(const Geom3<T> &, int, int64_t, const T *const *,          \
                                       const T *const *, T *const *, ndconv_fft_processor *,      \
                                       cudaStream_t, int);                                         \
    template size_t conv_fft_scratch_bytes<T>(const Geom3<T> &, int);                              \
    template int conv_fft_bake<T>(const Geom3<T> &, int, const T *, ndconv_fft_processor *, cudaStream_t);
NDCONV_INST_FFT(float)
NDCONV_INST_FFT(double)
NDCONV_INST_FFT(c32)
NDCONV_INST_FFT(c64)

// ---------------------------------------------------- processor forward --
// Natural-layout N-d transform of a contiguous array, then the reference's
// rotated layout (axes rotated right after each pass = the transpose of
// [d0] x [rest] for rank >= 2).
template <typename T>
int proc_forward(ndconv_fft_processor *proc, int rank, const int64_t *shape, const T *in,
                 typename CplxT<typename Elem<T>::Real>::type *out, cudaStream_t st) {
    using R = typename Elem<T>::Real;
    using C = typename CplxT<R>::type;
    const bool real = !Elem<T>::kComplex;
    int64_t s3[3] = {1, 1, 1};
    for (int i = 0; i < rank; i++) s3[3 - rank + i] = shape[i];
    RowArgs<T> r{};
    int s = row_plan<T>(s3[2], real, r);
    if (s) return s;
    const int64_t H = r.H;
    const size_t n = (size_t)s3[0] * s3[1] * H;
    Workspace ws{proc, st};
    void *base = nullptr;
    C *nat = out;
    if (rank >= 2) {
        if ((s = ws.get(sizeof(C) * n, &base))) return s;
        nat = reinterpret_cast<C *>(base);
    }
    r.mode = ROW_FWD_PLAIN;
    r.pin = in;
    r.n1 = s3[1];
    r.n_rows = s3[0] * s3[1];
    r.spec = nat;
    r.spec_s0 = s3[1] * H;
    r.spec_s1 = H;
    r.scale = 1;
    if ((s = launch_row(r, st))) return s;
    for (int a = 1; a >= 0; a--) {
        if (s3[a] <= 1) continue;
        ColArgs<C> c{};
        c.mode = COL_FWD;
        c.src = c.dst = nat;
        if ((s = plan_with_tw<C>(s3[a], c.pl, &c.tw))) return s;
        if (a == 1) {
            c.n_inner = H;
            c.n_outer = s3[0];
            c.src_outer = c.dst_outer = s3[1] * H;
            c.src_axis = c.dst_axis = H;
        } else {
            c.n_inner = s3[1] * H;
            c.n_outer = 1;
            c.src_axis = c.dst_axis = s3[1] * H;
        }
        c.valid_in = s3[a];
        if ((s = launch_col(c, st))) return s;
    }
    if (rank >= 2) {
        const int64_t rows = shape[0], cols = (int64_t)(n / shape[0]);
        dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
        transpose_kernel<C><<<grid, dim3(32, 8), 0, st>>>(nat, out, rows, cols);
        ndconv_count_launch();
        NDCONV_CUDA_OK(cudaGetLastError());
    }
    proc->rp_origin_len = shape[rank - 1];
    return NDCONV_OK;
}

template <typename T>
int proc_backward(ndconv_fft_processor *proc, int rank, const int64_t *spec_shape,
                  const typename CplxT<typename Elem<T>::Real>::type *in, T *out, int64_t *out_shape,
                  cudaStream_t st) {
    using R = typename Elem<T>::Real;
    using C = typename CplxT<R>::type;
    const bool real = !Elem<T>::kComplex;
    // natural shape: last axis of the rotated layout is d0
    int64_t nat_shape[3];
    if (rank == 1) nat_shape[0] = spec_shape[0];
    else {
        nat_shape[0] = spec_shape[rank - 1];
        for (int i = 1; i < rank; i++) nat_shape[i] = spec_shape[i - 1];
    }
    const int64_t H = nat_shape[rank - 1];
    const int64_t n_last = real ? proc->rp_origin_len : H;
    if (real && (n_last <= 0 || n_last / 2 + 1 != H))
        return ndconv_fail(NDCONV_ERR_INVALID, "spectrum does not match the last forward length");
    int64_t s3[3] = {1, 1, 1};
    for (int i = 0; i < rank; i++) s3[3 - rank + i] = nat_shape[i];
    size_t n = 1;
    for (int i = 0; i < rank; i++) n *= (size_t)nat_shape[i];
    Workspace ws{proc, st};
    void *base = nullptr;
    int s;
    if ((s = ws.get(sizeof(C) * n, &base))) return s;
    C *nat = reinterpret_cast<C *>(base);
    if (rank >= 2) {
        const int64_t rows = (int64_t)(n / nat_shape[0]), cols = nat_shape[0];
        dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
        transpose_kernel<C><<<grid, dim3(32, 8), 0, st>>>(in, nat, rows, cols);
        ndconv_count_launch();
        NDCONV_CUDA_OK(cudaGetLastError());
    } else {
        NDCONV_CUDA_OK(cudaMemcpyAsync(nat, in, sizeof(C) * n, cudaMemcpyDeviceToDevice, st));
    }
    for (int a = 0; a <= 1; a++) {
        if (s3[a] <= 1) continue;
        ColArgs<C> c{};
        c.mode = COL_INV;
        c.src = c.dst = nat;
        if ((s = plan_with_tw<C>(s3[a], c.pl, &c.tw))) return s;
        if (a == 1) {
            c.n_inner = H;
            c.n_outer = s3[0];
            c.src_outer = c.dst_outer = s3[1] * H;
            c.src_axis = c.dst_axis = H;
        } else {
            c.n_inner = s3[1] * H;
            c.n_outer = 1;
            c.src_axis = c.dst_axis = s3[1] * H;
        }
        c.valid_in = s3[a];
        c.crop_off = 0;
        c.crop_step = 1;
        c.n_out = s3[a];
        if ((s = launch_col(c, st))) return s;
    }
    RowArgs<T> r{};
    if ((s = row_plan<T>(n_last, real, r))) return s;
    r.mode = ROW_INV_PLAIN;
    r.pout = out;
    r.n1 = s3[1];
    r.n_rows = s3[0] * s3[1];
    r.spec = nat;
    r.spec_s0 = s3[1] * H;
    r.spec_s1 = H;
    double count = (double)n_last;
    for (int i = 0; i < rank - 1; i++) count *= (double)nat_shape[i];
    r.scale = (R)(1.0 / count);
    for (int i = 0; i < rank; i++) out_shape[i] = nat_shape[i];
    out_shape[rank - 1] = n_last;
    return launch_row(r, st);
}

#define NDCONV_INST_PROC(T)                                                                          \
    template int proc_forward<T>(ndconv_fft_processor *, int, const int64_t *, const T *,          \
                                 CplxT<Elem<T>::Real>::type *, cudaStream_t);                       \
    template int proc_backward<T>(ndconv_fft_processor *, int, const int64_t *,                     \
                                  const CplxT<Elem<T>::Real>::type *, T *, int64_t *, cudaStream_t);
NDCONV_INST_PROC(float)
NDCONV_INST_PROC(double)
NDCONV_INST_PROC(c32)
NDCONV_INST_PROC(c64)

}  // namespace ndconv

// ----------------------------------------------------- processor object --
extern "C" int ndconv_fft_processor_create(int32_t dtype, ndconv_fft_processor **out) {
    if (!out) return ndconv_fail(NDCONV_ERR_INVALID, "null output pointer");
    if (dtype != NDCONV_F32 && dtype != NDCONV_F64 && dtype != NDCONV_C32 && dtype != NDCONV_C64)
        return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "FFT processor needs f32/f64/c32/c64");
    auto *p = new ndconv_fft_processor{};
    p->dtype = dtype;
    cudaGetDevice(&p->device);
    *out = p;
    return NDCONV_OK;
}

extern "C" int ndconv_fft_processor_destroy(ndconv_fft_processor *p) {
    if (!p) return NDCONV_OK;
    if (p->ws || p->kbuf) cudaDeviceSynchronize();
    if (p->ws) cudaFree(p->ws);
    if (p->kbuf) cudaFree(p->kbuf);
    delete p;
    return NDCONV_OK;
}

int64_t ndconv_proc_origin_len(const ndconv_fft_processor *p) { return p->rp_origin_len; }
int32_t ndconv_proc_dtype(const ndconv_fft_processor *p) { return p->dtype; }

// ======================================================== batch plan ====
// A heterogeneous batch (instances with different shapes, kernels, modes,
// algorithms) executed by one persistent kernel.  Every instance becomes
// CTA-sized tasks: direct-convolution tiles, or the passes of its FFT
// convolution (one "level" per pass).  Tasks are stored in ticket order:
// all FFT tasks level-major across instances, then the direct tiles.  A CTA
// takes the next ticket, waits (bounded) until the previous level of the
// same instance has completed, runs the task and bumps its level counter.
// A task only waits for tasks with smaller tickets, which running CTAs have
// already claimed, so the queue always makes progress.
#include "direct_blocks.cuh"
#include "fold.h"
#include "fold_blocks.cuh"
#include "geometry.h"

namespace ndconv {
namespace batch {

enum TaskKind : int32_t {
    TK_DIRECT_SW = 1,
    TK_DIRECT_TILE4 = 2,
    TK_DIRECT_TILE1 = 3,
    TK_DIRECT_NAIVE = 4,
    TK_ROW_FWD_DATA = 10,
    TK_ROW_FWD_KERNEL = 11,
    TK_ROW_INV_OUT = 12,
    TK_ROW_FUSED = 13,
    TK_ROW_INV_MAC = 14,
    TK_COL = 20,
    TK_FOLD_SCAN = 30,  // axis-folding form: non-finite scan, chunk bx
    TK_FOLD_F1 = 31,    // first folded axis, chunk bx
    TK_FOLD_F0 = 32,    // second folded axis, chunk bx
    TK_FOLD_GEMM = 33,  // GEMM tile (bx, by)
};

// one instance of the axis-folding form inside the queue
struct FoldTaskArgs {
    FoldParams F;
    const float *x, *k;
    float *y, *W, *T1;
    int flag;  // index of its non-finite flag among the queue counters
    DirectParams<float> fb;
};
constexpr int64_t kFoldChunk = 256 * 8;  // elements per weight-folding / scan task

struct Task {
    int32_t kind, arg;
    int32_t bx, by, bz;
    int32_t done_ctr;   // counter bumped when done (-1: none)
    int32_t wait_ctr;   // counter to wait for (-1: none)
    int32_t wait_need;  // value it must reach
};

constexpr int kSpinLimit = 1 << 24;  // ~1-2 s of polling before giving up

__device__ __forceinline__ int ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// After the queue: instances whose skipped taps hold a non-finite weight
// get NaN everywhere, like the reference's sums.
__global__ void __launch_bounds__(256) batch_fixup_kernel(const DirectParams<float> *__restrict__ dargs,
                                                          const int *__restrict__ fix) {
    const DirectParams<float> &P = dargs[fix[blockIdx.y]];
    dead_tap_fixup_block<float>(P.k1, P.y1, P, blockIdx.x, gridDim.x);
}

// a separate function so that the GEMM tile's registers do not raise the
// other task kinds' register pressure
__device__ __noinline__ void fold_gemm_task(const FoldTaskArgs *A, int bx, int by, int *ctrs, unsigned char *smem) {
    foldk::gemm_tile<float>(A->x, A->W, A->y, A->F, ctrs + A->flag, A->k, A->fb, bx, by, smem, true);
}

__global__ void __launch_bounds__(256) persistent_kernel(const Task *__restrict__ tasks, int ntasks,
                                                         const RowArgs<float> *__restrict__ rargs,
                                                         const ColArgs<c32> *__restrict__ cargs,
                                                         const DirectParams<float> *__restrict__ dargs,
                                                         const FoldTaskArgs *__restrict__ fargs,
                                                         int *ctrs, int *ticket, int *status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_ticket;
    for (;;) {
        if (threadIdx.x == 0) s_ticket = atomicAdd(ticket, 1);
        __syncthreads();
        const int t = s_ticket;
        __syncthreads();
        if (t >= ntasks) return;
        const Task tk = tasks[t];
        if (tk.wait_ctr >= 0) {
            if (threadIdx.x == 0) {
                int it = 0;
                while (ld_acquire(ctrs + tk.wait_ctr) < tk.wait_need) {
                    if (++it > kSpinLimit) {
                        atomicOr(status, 1);  // dependency never completed: report, do not hang
                        break;
                    }
                    __nanosleep(64);
                }
            }
            __syncthreads();
        }
        switch (tk.kind) {
        case TK_DIRECT_SW: {
            const DirectParams<float> &P = dargs[tk.arg];
            direct_sw_block<float, 8, 16>(nullptr, nullptr, nullptr, P, tk.bx, tk.by, tk.bz, smem_raw);
            break;
        }
        case TK_DIRECT_TILE4: {
            const DirectParams<float> &P = dargs[tk.arg];
            direct_tile_block<float, 4>(nullptr, nullptr, nullptr, P, tk.bx, tk.by, tk.bz, smem_raw);
            break;
        }
        case TK_DIRECT_TILE1: {
            const DirectParams<float> &P = dargs[tk.arg];
            direct_tile_block<float, 1>(nullptr, nullptr, nullptr, P, tk.bx, tk.by, tk.bz, smem_raw);
            break;
        }
        case TK_DIRECT_NAIVE: {
            const DirectParams<float> &P = dargs[tk.arg];
            direct_naive_range<float>(P, (int64_t)tk.bx * 256 + threadIdx.x);
            break;
        }
        case TK_ROW_FWD_DATA: row_block<float, ROW_FWD_DATA>(rargs[tk.arg], tk.bx, 0, smem_raw); break;
        case TK_ROW_FWD_KERNEL: row_block<float, ROW_FWD_KERNEL>(rargs[tk.arg], tk.bx, 0, smem_raw); break;
        case TK_ROW_INV_OUT: row_block<float, ROW_INV_OUT>(rargs[tk.arg], tk.bx, 0, smem_raw); break;
        case TK_ROW_FUSED: row_block<float, ROW_FUSED>(rargs[tk.arg], tk.bx, 0, smem_raw); break;
        case TK_ROW_INV_MAC: row_block<float, ROW_INV_MAC>(rargs[tk.arg], tk.bx, 0, smem_raw); break;
        case TK_COL: {
            const ColArgs<c32> &A = cargs[tk.arg];
            col_block<c32>(A, tk.bx, tk.by, A.n_outer, 0, smem_raw);
            break;
        }
        case TK_FOLD_SCAN: {
            const FoldTaskArgs &A = fargs[tk.arg];
            const int64_t e = min((int64_t)(tk.bx + 1) * kFoldChunk, foldk::scan_count(A.F));
            bool bad = false;
            for (int64_t u = (int64_t)tk.bx * kFoldChunk + threadIdx.x; u < e; u += blockDim.x)
                bad |= foldk::scan_elem<float>(A.x, A.k, A.F, u);
            if (bad) atomicOr(ctrs + A.flag, 1);
            break;
        }
        case TK_FOLD_F1: {
            const FoldTaskArgs &A = fargs[tk.arg];
            const int64_t e = min((int64_t)(tk.bx + 1) * kFoldChunk, foldk::f1_count<float>(A.F));
            for (int64_t u = (int64_t)tk.bx * kFoldChunk + threadIdx.x; u < e; u += blockDim.x)
                foldk::f1_elem<float>(A.k, A.F, A.T1, u);
            break;
        }
        case TK_FOLD_F0: {
            const FoldTaskArgs &A = fargs[tk.arg];
            const int64_t e = min((int64_t)(tk.bx + 1) * kFoldChunk, foldk::f0_count<float>(A.F));
            for (int64_t u = (int64_t)tk.bx * kFoldChunk + threadIdx.x; u < e; u += blockDim.x)
                foldk::f0_elem<float>(A.T1, A.F, A.W, u, true);
            break;
        }
        case TK_FOLD_GEMM: fold_gemm_task(fargs + tk.arg, tk.bx, tk.by, ctrs, smem_raw); break;
        default: break;
        }
        __threadfence();  // this CTA's results visible GPU-wide before the counter moves
        __syncthreads();
        if (threadIdx.x == 0 && tk.done_ctr >= 0) atomicAdd(ctrs + tk.done_ctr, 1);
    }
}

// work estimate of one instance (for ordering direct tiles, longest first)
struct HostInst {
    int algo;        // 0 direct, 1 FFT
    int fv;          // FFT plan variant (FftVariant)
    int standalone;  // runs as ordinary launches before the persistent kernel
    int fold;        // f32 direct instance in the axis-folding form, inside the queue
    Plan3 P;
    const void *x, *k;
    void *y;
    size_t ws_off;   // workspace offset: spectra (FFT) or folded weights (direct)
    size_t ws_bytes; // direct: folded-form scratch (0: none)
    FftConvPlan<float> cp;
};

}  // namespace batch
}  // namespace ndconv

struct ndconv_batch_plan {
    int device = 0;
    int64_t n = 0;
    std::vector<ndconv::batch::HostInst> inst;
    std::vector<ndconv::batch::Task> tasks;
    std::vector<ndconv::RowArgs<float>> rargs;
    std::vector<ndconv::ColArgs<c32>> cargs;
    std::vector<ndconv::DirectParams<float>> dargs;
    std::vector<ndconv::batch::FoldTaskArgs> fargs;
    std::vector<int> fix;  // direct instances with skipped taps (non-finite fix-up after the queue)
    void *d_fix = nullptr;
    int64_t graph_kernels = 0;
    int nctrs = 0;
    size_t smem = 0;
    int grid = 0;
    void *d_tasks = nullptr, *d_rargs = nullptr, *d_cargs = nullptr, *d_dargs = nullptr, *d_fargs = nullptr;
    int *d_ctrs = nullptr;  // nctrs counters, then ticket, then status
    void *ws = nullptr;
    size_t ws_bytes = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t n_fft = 0, n_direct = 0, n_standalone = 0;
    cudaStream_t side = nullptr;  // ordinary launches beside the persistent kernel
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

namespace ndconv {
namespace batch {

constexpr size_t kBatchSmem = 100 * 1024;  // persistent kernel's shared memory (2 CTAs per SM)

template <typename V> int upload(const std::vector<V> &v, void **d) {
    const size_t bytes = sizeof(V) * (v.empty() ? 1 : v.size());
    NDCONV_CUDA_OK(cudaMalloc(d, bytes));
    if (!v.empty()) NDCONV_CUDA_OK(cudaMemcpy(*d, v.data(), sizeof(V) * v.size(), cudaMemcpyHostToDevice));
    return NDCONV_OK;
}

// Direct tiles of instance i as tasks; returns the shared memory a task needs.
size_t direct_tasks(ndconv_batch_plan *B, HostInst &h, std::vector<Task> &out) {
    DirectParams<float> D = h.P.direct<float>();
    D.xs = nullptr;
    D.ks = nullptr;
    D.ys = nullptr;
    D.x1 = static_cast<const float *>(h.x);
    D.k1 = static_cast<const float *>(h.k);
    D.y1 = static_cast<float *>(h.y);
    restrict_live_taps(D);
    permute_axes_for_tiles(D);
    const AxisGeom &A0 = D.g.ax[0], &A1 = D.g.ax[1], &A2 = D.g.ax[2];
    int kind = 0;
    int64_t gx = 0, gy = 0;
    if (plan_sw(D, 8) && smem_bytes(D) <= kBatchSmem) {
        kind = TK_DIRECT_SW;
        const int64_t TXo = sw_cols_per_cta(D, 8);
        gx = (A2.out + TXo - 1) / TXo;
        gy = (A1.out + D.sw_ty - 1) / D.sw_ty;
    } else {
        int BX, BY;
        if (plan_tile(D, 4, BX, BY) && smem_bytes(D) <= kBatchSmem) {
            kind = TK_DIRECT_TILE4;
            gx = (A2.out + (int64_t)BX * 4 - 1) / ((int64_t)BX * 4);
        } else if (plan_tile(D, 1, BX, BY) && smem_bytes(D) <= kBatchSmem) {
            kind = TK_DIRECT_TILE1;
            gx = (A2.out + BX - 1) / BX;
        } else {
            kind = TK_DIRECT_NAIVE;
        }
        if (kind != TK_DIRECT_NAIVE) gy = (A1.out + BY - 1) / BY;
    }
    const int arg = (int)B->dargs.size();
    B->dargs.push_back(D);
    if (taps_restricted(D)) B->fix.push_back(arg);
    if (kind == TK_DIRECT_NAIVE) {
        const int64_t total = A0.out * A1.out * A2.out;
        for (int64_t b = 0; b * 256 < total; b++) out.push_back(Task{kind, arg, (int32_t)b, 0, 0, -1, -1, 0});
        return 0;
    }
    for (int64_t z = 0; z < A0.out; z++)
        for (int64_t yy = 0; yy < gy; yy++)
            for (int64_t xx = 0; xx < gx; xx++)
                out.push_back(Task{kind, arg, (int32_t)xx, (int32_t)yy, (int32_t)z, -1, -1, 0});
    return smem_bytes(D);
}

}  // namespace batch
}  // namespace ndconv

namespace ndconv {
namespace batch {

// NDCONV_OK when every pass of the FFT form fits the kernels' limits
// (shared memory, grid), NDCONV_ERR_UNSUPPORTED otherwise.  Host only.
template <typename T> int fft_fits(const Geom3<T> &g, int fv) {
    using C = typename FftConvPlan<T>::C;
    FftConvPlan<T> cp;
    int s = make_conv_plan<T>(g, cp, fv);
    if (s) return s;
    return conv_fft_passes<T>(
        g, 0, cp, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0, 1, nullptr, nullptr,
        [&](RowArgs<T> &A, int) {
            int64_t grid;
            size_t sm;
            return A.n_rows > 0 ? prep_row(A, 1, grid, sm) : NDCONV_OK;
        },
        [&](ColArgs<C> &A, int) {
            int64_t gx, gy;
            size_t sm;
            return (A.n_outer > 0 && A.n_inner > 0) ? prep_col(A, gx, gy, sm) : NDCONV_OK;
        },
        [&](RowArgs<T> &A, RowArgs<T> &B, int) {
            int64_t grid;
            size_t sm;
            int r = A.n_rows > 0 ? prep_row(A, 1, grid, sm) : NDCONV_OK;
            return r ? r : (B.n_rows > 0 ? prep_row(B, 1, grid, sm) : NDCONV_OK);
        });
}

// Build the plan: per-instance tasks, spectra, device copies of everything.
// Device memory, graph, stream and events of a plan (null members skipped).
void release(ndconv_batch_plan *B) {
    if (B->exec) cudaGraphExecDestroy(B->exec);
    if (B->graph) cudaGraphDestroy(B->graph);
    cudaFree(B->d_tasks);
    cudaFree(B->d_rargs);
    cudaFree(B->d_cargs);
    cudaFree(B->d_dargs);
    cudaFree(B->d_fargs);
    cudaFree(B->d_fix);
    cudaFree(B->d_ctrs);
    cudaFree(B->ws);
    if (B->ev_fork) cudaEventDestroy(B->ev_fork);
    if (B->ev_join) cudaEventDestroy(B->ev_join);
    if (B->side) cudaStreamDestroy(B->side);
}

int create(const ndconv_problem *probs, int64_t n, const int32_t *algo, const void *const *data,
           const void *const *kernel, void *const *out, ndconv_batch_plan **outp) {
    auto *B = new ndconv_batch_plan();
    cudaGetDevice(&B->device);
    B->n = n;
    B->inst.resize((size_t)n);
    auto fail = [&](int st) {
        release(B);  // nothing of the plan has been launched yet
        delete B;
        return st;
    };
    // ---- pass 1: plans, algorithms, spectra sizes
    size_t ws = 0;
    for (int64_t i = 0; i < n; i++) {
        HostInst &h = B->inst[(size_t)i];
        const int32_t a = algo ? algo[i] : NDCONV_ALGO_FFT;
        if (a < 0 || a >= NDCONV_ALGO_COUNT || a == NDCONV_ALGO_DIRECT_BF16X3)
            return fail(ndconv_fail(NDCONV_ERR_INVALID, "algo must be 0 (direct), 1 (FFT) or 3..6 (FFT variants)"));
        h.algo = (a == NDCONV_ALGO_DIRECT) ? 0 : 1;
        h.fv = (a == NDCONV_ALGO_FFT_ND) ? FFTV_ND : (a == NDCONV_ALGO_FFT_RS) ? FFTV_RS
             : (a == NDCONV_ALGO_FFT_ND_POW2) ? FFTV_ND_POW2 : (a == NDCONV_ALGO_FFT_RS_POW2) ? FFTV_RS_POW2 : FFTV_AUTO;
        int s = plan_problem(&probs[i], h.algo, &h.P);
        if (s) {
            std::string m = "instance " + std::to_string(i) + ": " + ndconv_last_error();
            return fail(ndconv_fail(s, m.c_str()));
        }
        if (h.algo == 1 && (h.P.dtype == NDCONV_I32))
            return fail(ndconv_fail(NDCONV_ERR_UNSUPPORTED, "integer FFT convolution is not supported"));
        h.x = data[i];
        h.k = kernel[i];
        h.y = out[i];
        h.standalone = (h.P.dtype != NDCONV_F32);
        h.fold = 0;
        h.ws_off = 0;
        h.ws_bytes = 0;
        if (h.algo == 1) {
            // transforms that do not fit one CTA's shared memory: the same
            // convolution by the direct kernels (as ndconv_conv_fft does)
            int fs = NDCONV_OK;
            switch (h.P.dtype) {
            case NDCONV_F32: fs = fft_fits<float>(h.P.geom<float>(), h.fv); break;
            case NDCONV_F64: fs = fft_fits<double>(h.P.geom<double>(), h.fv); break;
            case NDCONV_C32: fs = fft_fits<c32>(h.P.geom<c32>(), h.fv); break;
            default: fs = fft_fits<c64>(h.P.geom<c64>(), h.fv); break;
            }
            if (fs == NDCONV_ERR_UNSUPPORTED) h.algo = 0;
            else if (fs) return fail(fs);
        }
        if (h.algo == 0) {
            // direct instances taken by the axis-folding form keep their
            // folded weights in the plan's workspace; f32 ones run as queue
            // tasks, others as ordinary launches
            switch (h.P.dtype) {
            case NDCONV_F32: h.ws_bytes = direct_scratch_bytes<float>(h.P.direct<float>()); break;
            case NDCONV_F64: h.ws_bytes = direct_scratch_bytes<double>(h.P.direct<double>()); break;
            case NDCONV_I32: h.ws_bytes = direct_scratch_bytes<int32_t>(h.P.direct<int32_t>()); break;
            case NDCONV_C32: h.ws_bytes = direct_scratch_bytes<c32>(h.P.direct<c32>()); break;
            default: h.ws_bytes = direct_scratch_bytes<c64>(h.P.direct<c64>()); break;
            }
            if (h.ws_bytes) {
                h.fold = !h.standalone;
                h.ws_off = ws;
                ws += (h.ws_bytes + 255) / 256 * 256;
            }
        }
        if (h.algo == 1 && !h.standalone) {
            if ((s = make_conv_plan<float>(h.P.geom<float>(), h.cp, h.fv))) return fail(s);
            h.ws_off = ws;
            ws += (sizeof(c32) * (h.cp.nK + h.cp.nS) + 255) / 256 * 256;
        }
    }
    // standalone FFT instances of other types get their own slice as scratch
    for (int64_t i = 0; i < n; i++) {
        HostInst &h = B->inst[(size_t)i];
        if (h.algo == 1 && h.standalone) {
            h.ws_off = ws;
            size_t b = 0;
            int s = NDCONV_OK;
            // plans now, so their twiddle tables exist before any graph capture
            switch (h.P.dtype) {
            case NDCONV_F64: {
                FftConvPlan<double> cp;
                s = make_conv_plan<double>(h.P.geom<double>(), cp, h.fv);
                b = conv_fft_scratch_bytes<double>(h.P.geom<double>(), h.fv);
                break;
            }
            case NDCONV_C32: {
                FftConvPlan<c32> cp;
                s = make_conv_plan<c32>(h.P.geom<c32>(), cp, h.fv);
                b = conv_fft_scratch_bytes<c32>(h.P.geom<c32>(), h.fv);
                break;
            }
            default: {
                FftConvPlan<c64> cp;
                s = make_conv_plan<c64>(h.P.geom<c64>(), cp, h.fv);
                b = conv_fft_scratch_bytes<c64>(h.P.geom<c64>(), h.fv);
                break;
            }
            }
            if (s) return fail(s);
            ws += (b + 255) / 256 * 256;
        }
    }
    B->ws_bytes = ws;
    if (ws) {
        cudaError_t e = cudaMalloc(&B->ws, ws);
        if (e != cudaSuccess) return fail(ndconv_fail(NDCONV_ERR_NO_MEMORY, cudaGetErrorString(e)));
    }
    // ---- pass 2: FFT passes as tasks (level-major across instances)
    struct Level {
        int64_t inst;
        int ctr;
        std::vector<Task> tasks;
    };
    std::vector<std::vector<Level>> per_inst((size_t)n);
    int max_levels = 0;
    for (int64_t i = 0; i < n; i++) {
        HostInst &h = B->inst[(size_t)i];
        if (h.algo != 1 || h.standalone) continue;
        c32 *Kh = reinterpret_cast<c32 *>(static_cast<unsigned char *>(B->ws) + h.ws_off);
        c32 *S = Kh + h.cp.nK;
        std::vector<Level> &lv = per_inst[(size_t)i];
        bool too_big = false, same_level = false;
        size_t inst_smem = 0;
        auto new_level = [&]() -> Level & {
            lv.push_back(Level{i, B->nctrs++, {}});
            return lv.back();
        };
        auto emit_row = [&](RowArgs<float> &A, int cnt) -> int {
            (void)cnt;
            if (A.n_rows <= 0) return NDCONV_OK;
            int64_t grid;
            size_t sm;
            int s2 = prep_row(A, 1, grid, sm);
            if (s2) return s2;
            if (sm > kBatchSmem) too_big = true;
            inst_smem = std::max(inst_smem, sm);
            const int arg = (int)B->rargs.size();
            A.l2only = 1;  // producers run in the same launch: no L1-cached reads
            B->rargs.push_back(A);
            int kind = TK_ROW_FWD_DATA;
            switch (A.mode) {
            case ROW_FWD_DATA: kind = TK_ROW_FWD_DATA; break;
            case ROW_FWD_KERNEL: kind = TK_ROW_FWD_KERNEL; break;
            case ROW_INV_OUT: kind = TK_ROW_INV_OUT; break;
            case ROW_INV_MAC: kind = TK_ROW_INV_MAC; break;
            default: kind = TK_ROW_FUSED; break;
            }
            Level &L = same_level ? lv.back() : new_level();
            for (int64_t b = 0; b < grid; b++) L.tasks.push_back(Task{kind, arg, (int32_t)b, 0, 0, L.ctr, -1, 0});
            return NDCONV_OK;
        };
        // independent passes share one level (one counter)
        auto emit_pair = [&](RowArgs<float> &A, RowArgs<float> &B2, int cnt) -> int {
            int s2 = emit_row(A, cnt);
            if (s2) return s2;
            same_level = !lv.empty();
            s2 = emit_row(B2, cnt);
            same_level = false;
            return s2;
        };
        auto emit_col = [&](ColArgs<c32> &A, int cnt) -> int {
            (void)cnt;
            if (A.n_outer <= 0 || A.n_inner <= 0) return NDCONV_OK;
            int64_t gx, gy;
            size_t sm;
            int s2 = prep_col(A, gx, gy, sm);
            if (s2) return s2;
            if (sm > kBatchSmem) too_big = true;
            inst_smem = std::max(inst_smem, sm);
            const int arg = (int)B->cargs.size();
            B->cargs.push_back(A);
            Level &L = new_level();
            for (int64_t o = 0; o < A.n_outer; o++)
                for (int64_t b = 0; b < gx; b++)
                    L.tasks.push_back(Task{TK_COL, arg, (int32_t)b, (int32_t)o, 0, L.ctr, -1, 0});
            return NDCONV_OK;
        };
        const Geom3<float> g = h.P.geom<float>();
        int s = conv_fft_passes<float>(g, h.P.reverse, h.cp, static_cast<const float *>(h.x),
                                       static_cast<const float *>(h.k), static_cast<float *>(h.y), nullptr,
                                       nullptr, nullptr, 0, 1, Kh, S, emit_row, emit_col, emit_pair);
        if (s) return fail(s);
        if (too_big) {
            // does not fit the persistent kernel's shared memory: ordinary launches
            h.standalone = 1;
            lv.clear();
            continue;
        }
        B->smem = std::max(B->smem, inst_smem);
        for (size_t l = 1; l < lv.size(); l++)
            for (Task &t : lv[l].tasks) {
                t.wait_ctr = lv[l - 1].ctr;
                t.wait_need = (int32_t)lv[l - 1].tasks.size();
            }
        max_levels = std::max(max_levels, (int)lv.size());
        B->n_fft++;
    }
    // ---- axis-folding instances: scan and first folding (level 0), second
    // folding (level 1), GEMM tiles (level 2)
    for (int64_t i = 0; i < n; i++) {
        HostInst &h = B->inst[(size_t)i];
        if (!h.fold) continue;
        DirectParams<float> full = h.P.direct<float>();
        full.xs = nullptr;
        full.ks = nullptr;
        full.ys = nullptr;
        full.x1 = static_cast<const float *>(h.x);
        full.k1 = static_cast<const float *>(h.k);
        full.y1 = static_cast<float *>(h.y);
        DirectParams<float> D = full;
        restrict_live_taps(D);
        FoldTaskArgs fa;
        if (!plan_fold(D, fa.F)) return fail(ndconv_fail(NDCONV_ERR_INVALID, "axis-folding plan changed"));
        const FoldParams &F = fa.F;
        fa.x = full.x1;
        fa.k = full.k1;
        fa.y = full.y1;
        fa.W = reinterpret_cast<float *>(static_cast<unsigned char *>(B->ws) + h.ws_off);
        fa.T1 = fa.W + F.cout * F.cin * F.km;
        {
            // tap tables, built here once and copied behind the folded weights
            int32_t *dtab = reinterpret_cast<int32_t *>(fa.T1 + F.km * F.ax[F.f0].K * F.ax[F.f1].out * F.ax[F.f1].n);
            const AxisGeom &G0 = F.ax[F.f0], &G1 = F.ax[F.f1];
            const int64_t e0 = fold_table_entries(G0), e1 = fold_table_entries(G1);
            std::vector<int32_t> tab((size_t)(e0 + e1));
            for (int64_t o = 0; o < G0.out; o++)
                fold_table_row(G0, o, tab.data() + o * (G0.n + 1), tab.data() + G0.out * (G0.n + 1) + o * G0.K);
            for (int64_t o = 0; o < G1.out; o++)
                fold_table_row(G1, o, tab.data() + e0 + o * (G1.n + 1), tab.data() + e0 + G1.out * (G1.n + 1) + o * G1.K);
            cudaError_t ce = cudaMemcpy(dtab, tab.data(), sizeof(int32_t) * tab.size(), cudaMemcpyHostToDevice);
            if (ce != cudaSuccess) return fail(ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(ce)));
            fold_set_tables(fa.F, dtab);
        }
        fa.flag = B->nctrs++;
        fa.fb = full;
        const int arg = (int)B->fargs.size();
        B->fargs.push_back(fa);
        std::vector<Level> &lv = per_inst[(size_t)i];
        auto chunks = [](int64_t cnt) { return (cnt + kFoldChunk - 1) / kFoldChunk; };
        lv.push_back(Level{i, B->nctrs++, {}});
        for (int64_t b = 0; b < chunks(foldk::scan_count(F)); b++)
            lv.back().tasks.push_back(Task{TK_FOLD_SCAN, arg, (int32_t)b, 0, 0, lv.back().ctr, -1, 0});
        for (int64_t b = 0; b < chunks(foldk::f1_count<float>(F)); b++)
            lv.back().tasks.push_back(Task{TK_FOLD_F1, arg, (int32_t)b, 0, 0, lv.back().ctr, -1, 0});
        lv.push_back(Level{i, B->nctrs++, {}});
        for (int64_t b = 0; b < chunks(foldk::f0_count<float>(F)); b++)
            lv.back().tasks.push_back(Task{TK_FOLD_F0, arg, (int32_t)b, 0, 0, lv.back().ctr, -1, 0});
        lv.push_back(Level{i, B->nctrs++, {}});
        const int64_t gx = (F.ax[F.m].out + foldk::FBM - 1) / foldk::FBM, gy = (F.cout + foldk::FBN - 1) / foldk::FBN;
        for (int64_t by = 0; by < gy; by++)
            for (int64_t bx = 0; bx < gx; bx++)
                lv.back().tasks.push_back(Task{TK_FOLD_GEMM, arg, (int32_t)bx, (int32_t)by, 0, lv.back().ctr, -1, 0});
        for (size_t l = 1; l < lv.size(); l++)
            for (Task &t : lv[l].tasks) {
                t.wait_ctr = lv[l - 1].ctr;
                t.wait_need = (int32_t)lv[l - 1].tasks.size();
            }
        max_levels = std::max(max_levels, (int)lv.size());
        B->smem = std::max(B->smem, foldk::gemm_smem<float>());
        B->n_direct++;
    }
    // ---- direct tiles, largest instances first, with a work estimate per task
    std::vector<std::pair<double, int64_t>> order;
    for (int64_t i = 0; i < n; i++) {
        HostInst &h = B->inst[(size_t)i];
        if (h.algo != 0 || h.standalone || h.fold) continue;
        const AxisGeom *A = h.P.ax;
        const double work = (double)(A[0].out * A[1].out * A[2].out) * (double)(A[0].K * A[1].K * A[2].K);
        order.push_back({-work, i});
    }
    std::sort(order.begin(), order.end());
    std::vector<Task> dtasks;
    std::vector<double> dwork;
    for (auto &o : order) {
        HostInst &h = B->inst[(size_t)o.second];
        const size_t before = dtasks.size();
        B->smem = std::max(B->smem, direct_tasks(B, h, dtasks));
        const size_t cnt = dtasks.size() - before;
        for (size_t t = 0; t < cnt; t++) dwork.push_back(-o.first / (double)(cnt ? cnt : 1));
        B->n_direct++;
    }
    // ---- queue order.  A task of FFT level l > 0 spins until level l - 1 of
    // its instance is done, so levels are separated by slices of direct work
    // (which never waits): the costliest direct tiles first (they set the
    // critical path), then level 0, a slice of direct tiles, level 1, ...
    {
        double total = 0;
        for (double w : dwork) total += w;
        size_t d = 0;
        double done = 0;
        auto take = [&](double upto) {
            while (d < dtasks.size() && done < upto) {
                B->tasks.push_back(dtasks[d]);
                done += dwork[d];
                d++;
            }
        };
        take(max_levels > 0 ? 0.25 * total : total);
        for (int l = 0; l < max_levels; l++) {
            for (int64_t i = 0; i < n; i++) {
                std::vector<Level> &lv = per_inst[(size_t)i];
                if ((int)lv.size() > l) B->tasks.insert(B->tasks.end(), lv[l].tasks.begin(), lv[l].tasks.end());
            }
            take(0.25 * total + 0.75 * total * (double)(l + 1) / (double)max_levels);
        }
        take(total * 2 + 1);
    }
    for (auto &h : B->inst) B->n_standalone += h.standalone;
    // ---- device copies
    int s;
    if ((s = upload(B->tasks, &B->d_tasks)) || (s = upload(B->rargs, &B->d_rargs)) ||
        (s = upload(B->cargs, &B->d_cargs)) || (s = upload(B->dargs, &B->d_dargs)) ||
        (s = upload(B->fargs, &B->d_fargs)) || (s = upload(B->fix, &B->d_fix)))
        return fail(s);
    {
        cudaError_t e = cudaMalloc((void **)&B->d_ctrs, sizeof(int) * (size_t)(B->nctrs + 2));
        if (e != cudaSuccess) return fail(ndconv_fail(NDCONV_ERR_NO_MEMORY, cudaGetErrorString(e)));
    }
    if (B->smem < 16) B->smem = 16;
    if (B->smem > kBatchSmem) return fail(ndconv_fail(NDCONV_ERR_INVALID, "batch task shared memory above the cap"));
    {
        cudaError_t e = ndconv_allow_smem((const void *)persistent_kernel, (int)kBatchSmem);
        if (e != cudaSuccess) return fail(ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e)));
        int per_sm = 0, sms = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persistent_kernel, 256, B->smem);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, B->device);
        if (e != cudaSuccess) return fail(ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e)));
        B->grid = std::max(1, per_sm) * sms;
        if ((int64_t)B->grid > (int64_t)B->tasks.size()) B->grid = (int)std::max<size_t>(1, B->tasks.size());
    }
    if (B->n_standalone > 0) {
        cudaError_t e = cudaStreamCreateWithFlags(&B->side, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B->ev_fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B->ev_join, cudaEventDisableTiming);
        if (e != cudaSuccess) return fail(ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e)));
    }
    *outp = B;
    return NDCONV_OK;
}

// Instances that run as ordinary launches (other element types, or FFT
// passes too large for the persistent kernel), on stream st.
int run_standalone(ndconv_batch_plan *B, cudaStream_t st) {
    for (auto &h : B->inst) {
        if (!h.standalone) continue;
        unsigned char *scr = static_cast<unsigned char *>(B->ws) + h.ws_off;
        int s = NDCONV_OK;
        if (h.algo == 0) {
            cudaError_t e = cudaSuccess;
            void *ds = h.ws_bytes ? scr : nullptr;
            const size_t db = h.ws_bytes;
            switch (h.P.dtype) {
            case NDCONV_F32: e = direct_conv_launch<float>((const float *)h.x, (const float *)h.k, (float *)h.y, h.P.direct<float>(), st, 0, ds, db); break;
            case NDCONV_F64: e = direct_conv_launch<double>((const double *)h.x, (const double *)h.k, (double *)h.y, h.P.direct<double>(), st, 0, ds, db); break;
            case NDCONV_I32: e = direct_conv_launch<int32_t>((const int32_t *)h.x, (const int32_t *)h.k, (int32_t *)h.y, h.P.direct<int32_t>(), st, 0, ds, db); break;
            case NDCONV_C32: e = direct_conv_launch<c32>((const c32 *)h.x, (const c32 *)h.k, (c32 *)h.y, h.P.direct<c32>(), st, 0, ds, db); break;
            default: e = direct_conv_launch<c64>((const c64 *)h.x, (const c64 *)h.k, (c64 *)h.y, h.P.direct<c64>(), st, 0, ds, db); break;
            }
            if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
            continue;
        }
        switch (h.P.dtype) {
        case NDCONV_F32: {
            const size_t b = sizeof(c32) * (h.cp.nK + h.cp.nS) + 256;
            s = conv_fft_run<float>(h.P.geom<float>(), h.P.reverse, (const float *)h.x, (const float *)h.k, (float *)h.y, nullptr, st, scr, b, h.fv);
            break;
        }
        case NDCONV_F64: s = conv_fft_run<double>(h.P.geom<double>(), h.P.reverse, (const double *)h.x, (const double *)h.k, (double *)h.y, nullptr, st, scr, conv_fft_scratch_bytes<double>(h.P.geom<double>(), h.fv), h.fv); break;
        case NDCONV_C32: s = conv_fft_run<c32>(h.P.geom<c32>(), h.P.reverse, (const c32 *)h.x, (const c32 *)h.k, (c32 *)h.y, nullptr, st, scr, conv_fft_scratch_bytes<c32>(h.P.geom<c32>(), h.fv), h.fv); break;
        default: s = conv_fft_run<c64>(h.P.geom<c64>(), h.P.reverse, (const c64 *)h.x, (const c64 *)h.k, (c64 *)h.y, nullptr, st, scr, conv_fft_scratch_bytes<c64>(h.P.geom<c64>(), h.fv), h.fv); break;
        }
        if (s) return s;
    }
    return NDCONV_OK;
}

// One execution: reset the queue, standalone instances, persistent kernel.
int enqueue(ndconv_batch_plan *B, cudaStream_t st) {
    NDCONV_CUDA_OK(cudaMemsetAsync(B->d_ctrs, 0, sizeof(int) * (size_t)(B->nctrs + 2), st));
    // ordinary launches (other element types, folded and oversized instances)
    // on a side stream, forked from and joined back into st, so they run
    // beside the persistent kernel instead of before it
    const bool side = B->n_standalone > 0 && B->side && B->ev_fork && B->ev_join;
    if (side) {
        NDCONV_CUDA_OK(cudaEventRecord(B->ev_fork, st));
        NDCONV_CUDA_OK(cudaStreamWaitEvent(B->side, B->ev_fork, 0));
    }
    int s = run_standalone(B, side ? B->side : st);
    if (s) return s;
    if (side) NDCONV_CUDA_OK(cudaEventRecord(B->ev_join, B->side));
    if (!B->tasks.empty()) {
        persistent_kernel<<<B->grid, 256, B->smem, st>>>(
            (const Task *)B->d_tasks, (int)B->tasks.size(), (const RowArgs<float> *)B->d_rargs,
            (const ColArgs<c32> *)B->d_cargs, (const DirectParams<float> *)B->d_dargs,
            (const FoldTaskArgs *)B->d_fargs, B->d_ctrs, B->d_ctrs + B->nctrs, B->d_ctrs + B->nctrs + 1);
        ndconv_count_launch();
        NDCONV_CUDA_OK(cudaGetLastError());
    }
    if (side) NDCONV_CUDA_OK(cudaStreamWaitEvent(st, B->ev_join, 0));
    if (!B->fix.empty()) {
        // parts per instance: kernel rows over 8 CTAs at most
        batch_fixup_kernel<<<dim3(8, (unsigned)B->fix.size()), 256, 0, st>>>((const DirectParams<float> *)B->d_dargs,
                                                                             (const int *)B->d_fix);
        ndconv_count_launch();
        NDCONV_CUDA_OK(cudaGetLastError());
    }
    return NDCONV_OK;
}

}  // namespace batch
}  // namespace ndconv

extern "C" int ndconv_batch_create(const ndconv_problem *problems, int64_t n, const int32_t *algo,
                                   const void *const *data, const void *const *kernel, void *const *out,
                                   ndconv_batch_plan **plan) {
    if (!problems || !data || !kernel || !out || !plan || n < 0)
        return ndconv_fail(NDCONV_ERR_INVALID, "null argument or negative count");
    return ndconv::batch::create(problems, n, algo, data, kernel, out, plan);
}

extern "C" int ndconv_batch_run(ndconv_batch_plan *B, int32_t use_graph, void *stream) {
    if (!B) return ndconv_fail(NDCONV_ERR_INVALID, "null plan");
    cudaStream_t st = (cudaStream_t)stream;
    if (!use_graph) return ndconv::batch::enqueue(B, st);
    if (!B->exec) {
        // capture once on a private stream, replay with cudaGraphLaunch
        cudaStream_t cs;
        NDCONV_CUDA_OK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        int s = NDCONV_OK;
        const uint64_t before = ndconv_kernel_launches();
        if (e == cudaSuccess) s = ndconv::batch::enqueue(B, cs);
        B->graph_kernels = (int64_t)(ndconv_kernel_launches() - before);
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(cs, &g);
        cudaStreamDestroy(cs);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        if (s) {
            cudaGraphDestroy(g);
            return s;
        }
        e = cudaGraphInstantiate(&B->exec, g, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
        }
        B->graph = g;
    }
    NDCONV_CUDA_OK(cudaGraphLaunch(B->exec, st));
    ndconv_count_launch((uint64_t)B->graph_kernels);  // the graph's kernels run again
    return NDCONV_OK;
}

extern "C" int ndconv_batch_run_plain(ndconv_batch_plan *B, void *stream) {
    // the plain drop-in: every instance through its own per-instance entry point
    if (!B) return ndconv_fail(NDCONV_ERR_INVALID, "null plan");
    cudaStream_t st = (cudaStream_t)stream;
    for (auto &h : B->inst) {
        unsigned char *scr = static_cast<unsigned char *>(B->ws) + h.ws_off;
        if (h.algo == 0) {
            cudaError_t e = cudaSuccess;
            switch (h.P.dtype) {
            case NDCONV_F32: e = ndconv::direct_conv_launch<float>((const float *)h.x, (const float *)h.k, (float *)h.y, h.P.direct<float>(), st, 0); break;
            case NDCONV_F64: e = ndconv::direct_conv_launch<double>((const double *)h.x, (const double *)h.k, (double *)h.y, h.P.direct<double>(), st, 0); break;
            case NDCONV_I32: e = ndconv::direct_conv_launch<int32_t>((const int32_t *)h.x, (const int32_t *)h.k, (int32_t *)h.y, h.P.direct<int32_t>(), st, 0); break;
            case NDCONV_C32: e = ndconv::direct_conv_launch<c32>((const c32 *)h.x, (const c32 *)h.k, (c32 *)h.y, h.P.direct<c32>(), st, 0); break;
            default: e = ndconv::direct_conv_launch<c64>((const c64 *)h.x, (const c64 *)h.k, (c64 *)h.y, h.P.direct<c64>(), st, 0); break;
            }
            if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
            continue;
        }
        int s;
        switch (h.P.dtype) {
        case NDCONV_F32: s = ndconv::conv_fft_run<float>(h.P.geom<float>(), h.P.reverse, (const float *)h.x, (const float *)h.k, (float *)h.y, nullptr, st, scr, sizeof(c32) * (h.cp.nK + h.cp.nS) + 256, h.fv); break;
        case NDCONV_F64: s = ndconv::conv_fft_run<double>(h.P.geom<double>(), h.P.reverse, (const double *)h.x, (const double *)h.k, (double *)h.y, nullptr, st, scr, ndconv::conv_fft_scratch_bytes<double>(h.P.geom<double>(), h.fv), h.fv); break;
        case NDCONV_C32: s = ndconv::conv_fft_run<c32>(h.P.geom<c32>(), h.P.reverse, (const c32 *)h.x, (const c32 *)h.k, (c32 *)h.y, nullptr, st, scr, ndconv::conv_fft_scratch_bytes<c32>(h.P.geom<c32>(), h.fv), h.fv); break;
        default: s = ndconv::conv_fft_run<c64>(h.P.geom<c64>(), h.P.reverse, (const c64 *)h.x, (const c64 *)h.k, (c64 *)h.y, nullptr, st, scr, ndconv::conv_fft_scratch_bytes<c64>(h.P.geom<c64>(), h.fv), h.fv); break;
        }
        if (s) return s;
    }
    return NDCONV_OK;
}

extern "C" int ndconv_batch_status(ndconv_batch_plan *B, void *stream) {
    if (!B) return ndconv_fail(NDCONV_ERR_INVALID, "null plan");
    int v = 0;
    NDCONV_CUDA_OK(cudaMemcpyAsync(&v, B->d_ctrs + B->nctrs + 1, sizeof(int), cudaMemcpyDeviceToHost,
                                   (cudaStream_t)stream));
    NDCONV_CUDA_OK(cudaStreamSynchronize((cudaStream_t)stream));
    if (v) return ndconv_fail(NDCONV_ERR_TIMEOUT, "a batch task waited too long for its predecessors");
    return NDCONV_OK;
}

extern "C" int ndconv_batch_info(const ndconv_batch_plan *B, int64_t info[8]) {
    if (!B || !info) return ndconv_fail(NDCONV_ERR_INVALID, "null argument");
    info[0] = (int64_t)B->tasks.size();
    info[1] = B->grid;
    info[2] = (int64_t)B->smem;
    info[3] = B->n_fft;
    info[4] = B->n_direct;
    info[5] = B->n_standalone;
    info[6] = (int64_t)B->ws_bytes;
    info[7] = B->nctrs;
    return NDCONV_OK;
}

extern "C" int ndconv_batch_destroy(ndconv_batch_plan *B) {
    if (!B) return NDCONV_OK;
    cudaDeviceSynchronize();
    ndconv::batch::release(B);
    delete B;
    return NDCONV_OK;
}

// ------------------------------------------------ plan facts / cost model --
// Modelled cost of one instance under each algorithm, used by the default
// dispatcher and as features of the learned one.  Rates are round numbers
// for one GB300 (FP32 FMA ~40 T/s, shared memory ~40 TB/s, HBM ~6.8 TB/s);
// the autotuner's measurements replace them where available.
extern "C" int ndconv_plan_info(const ndconv_problem *p, double out[8]) {
    using namespace ndconv;
    if (!out) return ndconv_fail(NDCONV_ERR_INVALID, "null output");
    for (int i = 0; i < 8; i++) out[i] = 0;
    Plan3 P;
    int s = plan_problem(p, 0, &P);
    if (s) return s;
    const AxisGeom *A = P.ax;
    const double nout = (double)(A[0].out * A[1].out * A[2].out);
    const double nx = (double)(A[0].n * A[1].n * A[2].n);
    double taps = (double)(A[0].K * A[1].K * A[2].K);
    double sw_slots = -1;  // issue slots of the sliding-window kernel, if it applies
    double fold_macs = -1, fold_prep = 0;  // the axis-folding form's GEMM and weight folding, if it applies
    {
        // the direct kernels only loop over taps that can see data
        DirectParams<float> D = P.direct<float>();
        restrict_live_taps(D);
        taps = (double)(D.t_n[0] * D.t_n[1] * D.t_n[2]);
        FoldParams F;
        if (plan_fold(D, F)) {
            const AxisGeom *FA = F.ax;
            fold_macs = (double)FA[F.m].out * (double)F.cout * (double)F.cin * (double)F.km;
            fold_prep = (double)F.km * FA[F.f0].K * FA[F.f1].out * FA[F.f1].n * FA[F.f1].K +
                        (double)F.cout * F.cin * F.km * FA[F.f0].K;
        }
        permute_axes_for_tiles(D);
        if (plan_sw(D, 8)) sw_slots = sw_cost(D, 8, 16);
    }
    const int es = (P.dtype == NDCONV_F64 || P.dtype == NDCONV_C32) ? 8 : (P.dtype == NDCONV_C64 ? 16 : 4);
    const double bytes = es * (nx + taps + nout);
    const double macs = nout * taps * ((P.dtype == NDCONV_C32 || P.dtype == NDCONV_C64) ? 4 : 1);
    // direct, seconds: FMA rate, or the sliding-window issue model (152 SMs x
    // 4 schedulers x ~1.9 GHz) when that kernel applies; other tilings run
    // at about a third of the FMA rate
    const double issue = 152.0 * 4 * 1.9e9;
    const double t_fma = (sw_slots >= 0) ? (sw_slots / issue > macs / 40e12 ? sw_slots / issue : macs / 40e12)
                                         : 3.0 * macs / 40e12;
    out[0] = t_fma + bytes / 6.8e12 + 4e-6;
    out[2] = macs;
    if (fold_macs >= 0) {
        // the direct entry point takes the axis-folding form: a gathered
        // CUDA-core GEMM (~10 T multiply-adds/s) after the weight folding
        const double cm = (P.dtype == NDCONV_C32 || P.dtype == NDCONV_C64) ? 4 : 1;
        out[0] = cm * fold_macs / 10e12 + fold_prep / 2e12 + bytes / 6.8e12 + 10e-6;
        out[2] = cm * fold_macs;
    }
    out[3] = bytes;
    // FFT: sizes, shared-memory fit, smem-traffic model
    const bool real = !(P.dtype == NDCONV_C32 || P.dtype == NDCONV_C64);
    int64_t F[3];
    for (int a = 0; a < 3; a++) F[a] = (A[a].L == 1) ? 1 : smooth_size(A[a].L, real && a == 2);
    out[4] = (double)F[0];
    out[5] = (double)F[1];
    out[6] = (double)F[2];
    const int csz = (P.dtype == NDCONV_F64 || P.dtype == NDCONV_C64) ? 16 : 8;
    const double budget = 100.0 * 1024;  // persistent kernel share
    if (P.dtype == NDCONV_I32) {
        out[1] = 1e30;
        out[7] = 0;
        return NDCONV_OK;
    }
    // rows too long for one CTA: overlap-save segments of the row-spectral form
    int64_t sn = 1, sl = 0;
    int64_t M = real ? F[2] / 2 : F[2];
    bool rs = false;
    if ((double)csz * 2 * (M + 1) * 1.07 > budget) {
        bool ok = false;
        switch (P.dtype) {
        case NDCONV_F32: ok = seg_plan<float>(A[2], false, F[2], sn, sl); break;
        case NDCONV_F64: ok = seg_plan<double>(A[2], false, F[2], sn, sl); break;
        case NDCONV_C32: ok = seg_plan<c32>(A[2], false, F[2], sn, sl); break;
        default: ok = seg_plan<c64>(A[2], false, F[2], sn, sl); break;
        }
        if (!ok) {
            out[1] = 1e30;
            out[7] = 0;
            return NDCONV_OK;
        }
        out[6] = (double)F[2];
        M = real ? F[2] / 2 : F[2];
        rs = true;
    }
    for (int a = 0; a < 2; a++)
        if (!rs && F[a] > 1 && (double)csz * 2 * F[a] * 1.07 > budget) {
            out[1] = 1e30;  // columns too long for the N-d form: conv_fft runs the direct kernels
            out[7] = 0;
            return NDCONV_OK;
        }
    auto stages = [](int64_t L) {
        FftPlanDev pl;
        if (L <= 1 || !make_plan((int)L, pl)) return 0.0;
        double c = 0;
        for (int i = 0; i < pl.nst; i++) c += 1.0;
        return c;
    };
    const double H = real ? (double)(F[2] / 2 + 1) : (double)F[2];
    const double dram_base = bytes;
    if (rs && (A[0].L > 1 || A[1].L > 1 || sn > 1)) {
        // row transforms (data rows and segments, kernel rows, output rows)
        // plus the spectral tap sums through L2
        const double rows = (double)A[0].L * A[1].L * sn + (double)A[0].K * A[1].K + (double)A[0].out * A[1].out * sn;
        const double smem_bytes = rows * H * (stages(M) + 1) * 16.0;
        const double mac_bytes = (double)A[0].out * A[1].out * sn * H * (double)(A[0].K * A[1].K) * 2.0 * csz;
        const double dram = dram_base + 2.0 * (double)A[0].L * A[1].L * sn * H * csz;
        out[1] = smem_bytes / 40e12 + mac_bytes / 20e12 + dram / 6.8e12 + 12e-6;
        out[7] = 1;
        return NDCONV_OK;
    }
    const double vol = (double)F[0] * F[1] * H;  // spectrum elements
    // kernel + data forward, inverse: ~3 transforms, each stage a smem round trip (16 B/elem)
    const double st = stages(M) + stages(F[1]) + stages(F[0]) + 1;
    const double smem_bytes = 3.0 * vol * st * 16.0;
    const double dram = dram_base + 4.0 * vol * csz;
    out[1] = smem_bytes / 40e12 + dram / 6.8e12 + 12e-6;
    out[7] = 1;
    return NDCONV_OK;
}
