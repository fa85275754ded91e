// Shared-memory FFT building blocks (sm_103a).
//
// A CTA transforms nb transforms of length L held in shared memory with
// element (b, i) at slot sx(i * nb + b) (nb a power of two).  Each stage is a
// Stockham autosort radix-R step (no bit reversal), ping-ponging between
// two buffers: butterfly j reads buf[j + r L/R], applies the twiddles
// w^(r * (j mod Ns)) with w = exp(-+2 pi i / (Ns R)), does a radix-R DFT in
// registers and writes to (j / Ns) Ns R + (j mod Ns) + r Ns.  After all
// stages the result is in natural order.  Twiddles come from tables
// evaluated in FP64 on the GPU and rounded once: per stage, the rows
// w^(t r) (t < Ns, r < R) that one butterfly applies, loaded as vectors; the
// generic odd-prime stage uses tw[t] = exp(-2 pi i t / L).
#pragma once
#include "common.cuh"

namespace ndconv {

template <typename R> struct CplxT;
template <> struct CplxT<float> { using type = c32; };
template <> struct CplxT<double> { using type = c64; };

constexpr int kMaxStages = 24;
constexpr int kMaxGenericRadix = 64;

// n / d for n < 2^31 with a precomputed multiplier: q = umulhi(n, m) >> s
// (m = ceil(2^(31+t) / d), s = t - 1, t = ceil(log2 d) >= 1; d == 1 is the
// identity).  Exact for all n < 2^31 because d <= 2^t.
struct FastDiv {
    uint32_t d, m, s;
};
inline FastDiv make_fastdiv(uint32_t d) {
    FastDiv f{d, 0, 0};
    if (d <= 1) return f;
    uint32_t t = 0;
    while ((1ull << t) < d) t++;
    f.m = (uint32_t)(((1ull << (31 + t)) + d - 1) / d);
    f.s = t - 1;
    return f;
}
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv &f) {
    return f.d == 1 ? n : (__umulhi(n, f.m) >> f.s);
}

struct FftPlanDev {
    int L;
    int nst;
    int rad[kMaxStages];
    FastDiv ns[kMaxStages];  // Ns (product of the previous radices) per stage
    // stage twiddle table: stage s >= 1 holds the Ns x R entries
    // w^(t r), w = exp(-2 pi i / (Ns R)), at tws[twoff[s] + t R + r]
    // (twoff even, so that bin pairs load as one 16-byte vector)
    int twoff[kMaxStages];
    int twn;          // entries of the table
    const void *tws;  // the table on the device (element type of the transform)
};

// Shared-memory slot of logical element u: one padding slot after every
// 128-byte wavefront (16 c32 or 8 c64 values), so the stride-R stores of
// the first Stockham stages spread over all banks.
template <typename C> __host__ __device__ __forceinline__ int sx(int u) {
    return u + (u >> (sizeof(C) <= 8 ? 4 : 3));
}
// slots needed for n logical elements
template <typename C> __host__ __device__ __forceinline__ int64_t padded_slots(int64_t n) {
    return n + (n >> (sizeof(C) <= 8 ? 4 : 3)) + 1;
}

// Load a complex value past L1 (other CTAs of the same launch may have
// written it).
__device__ __forceinline__ float fmaf_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmaf_t(double a, double b, double c) { return fma(a, b, c); }

// read-only (L1-cached) load of data written by an earlier launch
template <typename C> __device__ __forceinline__ C ldg_c(const C *p) {
    if constexpr (sizeof(C) == 8) {
        const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
        return C{v.x, v.y};
    } else {
        const double2 v = __ldg(reinterpret_cast<const double2 *>(p));
        return C{v.x, v.y};
    }
}
template <typename C> __device__ __forceinline__ C ldcg_c(const C *p) {
    if constexpr (sizeof(C) == 8) {
        const float2 v = __ldcg(reinterpret_cast<const float2 *>(p));
        return C{v.x, v.y};
    } else {
        const double2 v = __ldcg(reinterpret_cast<const double2 *>(p));
        return C{v.x, v.y};
    }
}

template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    return C{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return C{a.re + b.re, a.im + b.im}; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return C{a.re - b.re, a.im - b.im}; }
template <typename C> __device__ __forceinline__ C cconj(C a) { return C{a.re, -a.im}; }
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename C> __device__ __forceinline__ C mul_mi(C a) {
    return INV ? C{-a.im, a.re} : C{a.im, -a.re};
}
template <typename C, typename R> __device__ __forceinline__ C cscale(C a, R s) { return C{a.re * s, a.im * s}; }

template <bool INV, typename C> __device__ __forceinline__ void dft2(C *v) {
    C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}
template <bool INV, typename C> __device__ __forceinline__ void dft4(C &a0, C &a1, C &a2, C &a3) {
    C s02 = cadd(a0, a2), d02 = csub(a0, a2), s13 = cadd(a1, a3), d13 = mul_mi<INV>(csub(a1, a3));
    a0 = cadd(s02, s13);
    a2 = csub(s02, s13);
    a1 = cadd(d02, d13);
    a3 = csub(d02, d13);
}
template <bool INV, typename C> __device__ __forceinline__ void dft3(C *v) {
    using R = decltype(v[0].re);
    const R h = (R)0.5, s = (R)0.86602540378443864676;  // cos(pi/3), sin(pi/3)
    C a0 = v[0], sum = cadd(v[1], v[2]), dif = csub(v[1], v[2]);
    C t = C{a0.re - h * sum.re, a0.im - h * sum.im};
    C u = mul_mi<INV>(cscale(dif, s));
    v[0] = cadd(a0, sum);
    v[1] = cadd(t, u);
    v[2] = csub(t, u);
}
template <bool INV, typename C> __device__ __forceinline__ void dft5(C *v) {
    using R = decltype(v[0].re);
    const R c1 = (R)0.30901699437494742410, c2 = (R)-0.80901699437494742410;  // cos(2pi/5), cos(4pi/5)
    const R s1 = (R)0.95105651629515357212, s2 = (R)0.58778525229247312917;   // sin(2pi/5), sin(4pi/5)
    C a0 = v[0];
    C b1 = cadd(v[1], v[4]), b2 = cadd(v[2], v[3]), d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
    C t1 = C{a0.re + c1 * b1.re + c2 * b2.re, a0.im + c1 * b1.im + c2 * b2.im};
    C t2 = C{a0.re + c2 * b1.re + c1 * b2.re, a0.im + c2 * b1.im + c1 * b2.im};
    C u1 = mul_mi<INV>(C{s1 * d1.re + s2 * d2.re, s1 * d1.im + s2 * d2.im});
    C u2 = mul_mi<INV>(C{s2 * d1.re - s1 * d2.re, s2 * d1.im - s1 * d2.im});
    v[0] = cadd(a0, cadd(b1, b2));
    v[1] = cadd(t1, u1);
    v[4] = csub(t1, u1);
    v[2] = cadd(t2, u2);
    v[3] = csub(t2, u2);
}
template <bool INV, typename C> __device__ __forceinline__ void dft7(C *v) {
    using R = decltype(v[0].re);
    // cos / sin of 2 pi k / 7, k = 1..3
    const R c1 = (R)0.62348980185873353053, c2 = (R)-0.22252093395631440429, c3 = (R)-0.90096886790241912624;
    const R s1 = (R)0.78183148246802980871, s2 = (R)0.97492791218182360702, s3 = (R)0.43388373911755812048;
    const C a0 = v[0];
    const C b1 = cadd(v[1], v[6]), b2 = cadd(v[2], v[5]), b3 = cadd(v[3], v[4]);
    const C d1 = csub(v[1], v[6]), d2 = csub(v[2], v[5]), d3 = csub(v[3], v[4]);
    const C t1 = C{a0.re + c1 * b1.re + c2 * b2.re + c3 * b3.re, a0.im + c1 * b1.im + c2 * b2.im + c3 * b3.im};
    const C t2 = C{a0.re + c2 * b1.re + c3 * b2.re + c1 * b3.re, a0.im + c2 * b1.im + c3 * b2.im + c1 * b3.im};
    const C t3 = C{a0.re + c3 * b1.re + c1 * b2.re + c2 * b3.re, a0.im + c3 * b1.im + c1 * b2.im + c2 * b3.im};
    const C u1 = mul_mi<INV>(C{s1 * d1.re + s2 * d2.re + s3 * d3.re, s1 * d1.im + s2 * d2.im + s3 * d3.im});
    const C u2 = mul_mi<INV>(C{s2 * d1.re - s3 * d2.re - s1 * d3.re, s2 * d1.im - s3 * d2.im - s1 * d3.im});
    const C u3 = mul_mi<INV>(C{s3 * d1.re - s1 * d2.re + s2 * d3.re, s3 * d1.im - s1 * d2.im + s2 * d3.im});
    v[0] = cadd(a0, cadd(b1, cadd(b2, b3)));
    v[1] = cadd(t1, u1);
    v[6] = csub(t1, u1);
    v[2] = cadd(t2, u2);
    v[5] = csub(t2, u2);
    v[3] = cadd(t3, u3);
    v[4] = csub(t3, u3);
}
template <bool INV, typename C> __device__ __forceinline__ void dft8(C *v) {
    using R = decltype(v[0].re);
    const R r2 = (R)0.70710678118654752440;
    C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    C o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<INV>(e0, e1, e2, e3);
    dft4<INV>(o0, o1, o2, o3);
    // o_k *= w8^k, w8 = exp(-+ i pi / 4)
    o1 = INV ? C{r2 * (o1.re - o1.im), r2 * (o1.re + o1.im)} : C{r2 * (o1.re + o1.im), r2 * (o1.im - o1.re)};
    o2 = mul_mi<INV>(o2);
    o3 = INV ? C{-r2 * (o3.re + o3.im), r2 * (o3.re - o3.im)} : C{r2 * (o3.im - o3.re), -r2 * (o3.re + o3.im)};
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, o1);
    v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2);
    v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3);
    v[7] = csub(e3, o3);
}

// radix 10 = 2 x 5: X[k] = E[k] + w10^k O[k], X[k + 5] = E[k] - w10^k O[k]
// (E, O: 5-point transforms of the even and odd samples)
template <bool INV, typename C> __device__ __forceinline__ void dft10(C *v) {
    using R = decltype(v[0].re);
    C e[5], o[5];
#pragma unroll
    for (int m = 0; m < 5; m++) {
        e[m] = v[2 * m];
        o[m] = v[2 * m + 1];
    }
    dft5<INV>(e);
    dft5<INV>(o);
    // w10^k = exp(-+ 2 pi i k / 10), k = 1..4
    const R c1 = (R)0.80901699437494742410, s1 = (R)0.58778525229247312917;
    const R c2 = (R)0.30901699437494742410, s2 = (R)0.95105651629515357212;
    const R sg = INV ? (R)1 : (R)-1;
    const C w[5] = {C{1, 0}, C{c1, sg * s1}, C{c2, sg * s2}, C{-c2, sg * s2}, C{-c1, sg * s1}};
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const C t = (k == 0) ? o[0] : cmul(o[k], w[k]);
        v[k] = cadd(e[k], t);
        v[k + 5] = csub(e[k], t);
    }
}

// radix 16 = 4 x 4: four 4-point transforms over stride-4 samples, the
// twiddles w16^(n2 k1), four 4-point transforms across them; X[k1 + 4 k2]
template <bool INV, typename C> __device__ __forceinline__ void dft16(C *v) {
    using R = decltype(v[0].re);
    C y[4][4];
#pragma unroll
    for (int n2 = 0; n2 < 4; n2++) {
        C a0 = v[n2], a1 = v[n2 + 4], a2 = v[n2 + 8], a3 = v[n2 + 12];
        dft4<INV>(a0, a1, a2, a3);
        y[n2][0] = a0;
        y[n2][1] = a1;
        y[n2][2] = a2;
        y[n2][3] = a3;
    }
    // w16^m = exp(-+ 2 pi i m / 16) for the products m = n2 k1
    const R c = (R)0.92387953251128675613, s = (R)0.38268343236508977173, h = (R)0.70710678118654752440;
    const R sg = INV ? (R)1 : (R)-1;
    const C w1 = C{c, sg * s}, w2 = C{h, sg * h}, w3 = C{s, sg * c}, w6 = C{-h, sg * h}, w9 = C{-c, -sg * s};
    y[1][1] = cmul(y[1][1], w1);
    y[1][2] = cmul(y[1][2], w2);
    y[1][3] = cmul(y[1][3], w3);
    y[2][1] = cmul(y[2][1], w2);
    y[2][2] = mul_mi<INV>(y[2][2]);  // w16^4 = -+ i
    y[2][3] = cmul(y[2][3], w6);
    y[3][1] = cmul(y[3][1], w3);
    y[3][2] = cmul(y[3][2], w6);
    y[3][3] = cmul(y[3][3], w9);
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
        C a0 = y[0][k1], a1 = y[1][k1], a2 = y[2][k1], a3 = y[3][k1];
        dft4<INV>(a0, a1, a2, a3);
        v[k1] = a0;
        v[k1 + 4] = a1;
        v[k1 + 8] = a2;
        v[k1 + 12] = a3;
    }
}

template <bool INV, typename C>
__device__ __forceinline__ C twiddle(const C *__restrict__ tw, int e) {
    C w = tw[e];
    return INV ? cconj(w) : w;
}

// The R - 1 twiddles w^(t r), r = 1..R-1, of a butterfly from its row of the
// stage table (conjugated for the inverse).  Even radices load entry pairs
// as 16-byte vectors (the row's first entry, w^0, is loaded and unused).
template <bool INV, int RAD, typename C>
__device__ __forceinline__ void stage_twiddles(C (&w)[RAD], const C *__restrict__ row) {
    if constexpr (sizeof(C) == 8 && RAD % 2 == 0) {
        const float4 *p = reinterpret_cast<const float4 *>(row);
#pragma unroll
        for (int h = 0; h < RAD / 2; h++) {
            const float4 v = __ldg(p + h);
            w[2 * h] = C{v.x, INV ? -v.y : v.y};
            w[2 * h + 1] = C{v.z, INV ? -v.w : v.w};
        }
    } else {
#pragma unroll
        for (int r = 1; r < RAD; r++) {
            const C v = ldg_c(row + r);
            w[r] = INV ? cconj(v) : v;
        }
    }
}

// Geometry of one Stockham stage: transform length L, nb interleaved
// transforms (a power of two, lognb = log2 nb) and Ns, the product of the
// previous radices.  RtGeo holds them at run time; CtGeo fixes them at
// compile time for the lengths the row kernels specialise, so that the same
// stage code folds its index arithmetic into constants.
struct RtGeo {
    int L, nb, lognb;
    FastDiv nsd;
    __device__ __forceinline__ int ns() const { return (int)nsd.d; }
    __device__ __forceinline__ int div_ns(int j) const { return (int)fdiv((uint32_t)j, nsd); }
};
template <int L_, int NB_, int NS_> struct CtGeo {
    static_assert(NB_ == 1 || NB_ == 2 || NB_ == 4 || NB_ == 8, "rows per CTA: 1, 2, 4 or 8");
    static constexpr int L = L_, nb = NB_, lognb = NB_ == 1 ? 0 : NB_ == 2 ? 1 : NB_ == 4 ? 2 : 3;
    __device__ __forceinline__ static constexpr int ns() { return NS_; }
    __device__ __forceinline__ static constexpr int div_ns(int j) { return j / NS_; }
};

// One radix-R Stockham stage over nb interleaved transforms.  Butterfly j
// (of transform b) reads logical elements u + r si (u = j nb + b,
// si = (L / R) nb) and writes uo + r so (so = Ns nb).  When a stride is a
// multiple of the padded wavefront (16 c32 / 8 c64 elements), or a
// butterfly's outputs stay inside one wavefront, the padded slot of element
// r is the first one's plus r times a fixed step, so each access is one add
// away from the last.
template <bool INV, int RAD, typename C, typename Geo>
__device__ __forceinline__ void stockham_stage_g(const C *src, C *dst, const Geo &g, const C *__restrict__ tws) {
    const int Ns = g.ns();
    const int nr = g.L / RAD;
    const int total = nr << g.lognb;
    constexpr int kWf = sizeof(C) <= 8 ? 16 : 8;  // elements per padded wavefront (see sx)
    constexpr int kSh = sizeof(C) <= 8 ? 4 : 3;
    const int si = total, so = Ns << g.lognb;
    const bool lin_i = (si & (kWf - 1)) == 0;
    const bool lin_o = (so & (kWf - 1)) == 0 || (kWf % (RAD * so)) == 0;
    const int psi = si + (si >> kSh);                             // padded input step (lin_i)
    const int pso = (so & (kWf - 1)) == 0 ? so + (so >> kSh) : so;  // padded output step (lin_o)
#pragma unroll 2
    for (int u = threadIdx.x; u < total; u += blockDim.x) {
        const int b = u & (g.nb - 1);
        const int j = u >> g.lognb;
        const int q = g.div_ns(j);
        const int t = j - q * Ns;
        C v[RAD];
        if (lin_i) {
            const C *s0 = src + sx<C>(u);
#pragma unroll
            for (int r = 0; r < RAD; r++) v[r] = s0[r * psi];
        } else {
#pragma unroll
            for (int r = 0; r < RAD; r++) v[r] = src[sx<C>(u + r * si)];
        }
        if (t) {
            C w[RAD];
            stage_twiddles<INV, RAD>(w, tws + t * RAD);
#pragma unroll
            for (int r = 1; r < RAD; r++) v[r] = cmul(v[r], w[r]);
        }
        if constexpr (RAD == 2) dft2<INV>(v);
        else if constexpr (RAD == 3) dft3<INV>(v);
        else if constexpr (RAD == 4) dft4<INV>(v[0], v[1], v[2], v[3]);
        else if constexpr (RAD == 5) dft5<INV>(v);
        else if constexpr (RAD == 7) dft7<INV>(v);
        else if constexpr (RAD == 8) dft8<INV>(v);
        else if constexpr (RAD == 10) dft10<INV>(v);
        else if constexpr (RAD == 16) dft16<INV>(v);
        const int uo = ((q * Ns * RAD + t) << g.lognb) + b;
        if (lin_o) {
            C *d0 = dst + sx<C>(uo);
#pragma unroll
            for (int r = 0; r < RAD; r++) d0[r * pso] = v[r];
        } else {
#pragma unroll
            for (int r = 0; r < RAD; r++) dst[sx<C>(uo + r * so)] = v[r];
        }
    }
}

template <bool INV, int RAD, typename C>
__device__ __forceinline__ void stockham_stage(const C *src, C *dst, int L, int nb, int lognb,
                                               const FastDiv &nsd, const C *__restrict__ tws) {
    stockham_stage_g<INV, RAD>(src, dst, RtGeo{L, nb, lognb, nsd}, tws);
}

// Generic odd-prime radix (O(p^2), runtime p <= kMaxGenericRadix).
template <bool INV, typename C>
__device__ void stockham_stage_generic(const C *src, C *dst, int L, int nb, int lognb, const FastDiv &nsd,
                                       int RAD, const C *__restrict__ tw) {
    const int Ns = (int)nsd.d;
    const int nr = L / RAD;
    const int twstep = L / (Ns * RAD);
    const int wstep = L / RAD;  // tw index step for the radix's own roots
    const int total = nr << lognb;
    for (int u = threadIdx.x; u < total; u += blockDim.x) {
        const int b = u & (nb - 1);
        const int j = u >> lognb;
        const int q = (int)fdiv((uint32_t)j, nsd);
        const int t = j - q * Ns;
        C v[kMaxGenericRadix];
        for (int r = 0; r < RAD; r++) {
            C x = src[sx<C>(((j + r * nr) << lognb) + b)];
            if (t && r) x = cmul(x, twiddle<INV>(tw, t * r * twstep));
            v[r] = x;
        }
        const int base = q * Ns * RAD + t;
        for (int k = 0; k < RAD; k++) {
            C acc = v[0];
            for (int m = 1; m < RAD; m++) acc = cadd(acc, cmul(v[m], twiddle<INV>(tw, ((m * k) % RAD) * wstep)));
            dst[sx<C>(((base + k * Ns) << lognb) + b)] = acc;
        }
    }
}

// Full transform of nb interleaved length-L sequences starting in `a`, using
// `b` as the second buffer.  Returns the buffer holding the result.  Must be
// called by all threads of the CTA; ends with a barrier after every stage.
template <bool INV, typename C>
__device__ C *block_fft(C *a, C *b, int nb, int lognb, const FftPlanDev &pl, const C *__restrict__ tw) {
    C *src = a, *dst = b;
    const C *__restrict__ tws = static_cast<const C *>(pl.tws);
    for (int s = 0; s < pl.nst; s++) {
        const int R = pl.rad[s];
        const C *tr = tws + pl.twoff[s];
        switch (R) {
        case 2: stockham_stage<INV, 2>(src, dst, pl.L, nb, lognb, pl.ns[s], tr); break;
        case 3: stockham_stage<INV, 3>(src, dst, pl.L, nb, lognb, pl.ns[s], tr); break;
        case 4: stockham_stage<INV, 4>(src, dst, pl.L, nb, lognb, pl.ns[s], tr); break;
        case 5: stockham_stage<INV, 5>(src, dst, pl.L, nb, lognb, pl.ns[s], tr); break;
        case 7: stockham_stage<INV, 7>(src, dst, pl.L, nb, lognb, pl.ns[s], tr); break;
        case 8: stockham_stage<INV, 8>(src, dst, pl.L, nb, lognb, pl.ns[s], tr); break;
        case 10: stockham_stage<INV, 10>(src, dst, pl.L, nb, lognb, pl.ns[s], tr); break;
        case 16: stockham_stage<INV, 16>(src, dst, pl.L, nb, lognb, pl.ns[s], tr); break;
        default: stockham_stage_generic<INV>(src, dst, pl.L, nb, lognb, pl.ns[s], R, tw); break;
        }
        __syncthreads();
        C *tmp = src;
        src = dst;
        dst = tmp;
    }
    return src;
}

// The three-stage transform of a length whose plan (make_plan) is radices
// R0, R1, R2, over NB interleaved rows, with the geometry fixed at compile
// time: the same stages and twiddle tables as block_fft, so the results are
// the same.  Returns the buffer holding the result (b).
template <bool INV, int L, int NB, int R0, int R1, int R2, typename C>
__device__ C *block_fft_ct(C *a, C *b, const FftPlanDev &pl) {
    static_assert(R0 * R1 * R2 == L, "radices must multiply to the length");
    const C *__restrict__ tws = static_cast<const C *>(pl.tws);
    stockham_stage_g<INV, R0>(a, b, CtGeo<L, NB, 1>{}, tws + pl.twoff[0]);
    __syncthreads();
    stockham_stage_g<INV, R1>(b, a, CtGeo<L, NB, R0>{}, tws + pl.twoff[1]);
    __syncthreads();
    stockham_stage_g<INV, R2>(a, b, CtGeo<L, NB, R0 * R1>{}, tws + pl.twoff[2]);
    __syncthreads();
    return b;
}

}  // namespace ndconv
