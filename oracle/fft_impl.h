/*
 * Oracle FFT, instantiated once per precision by ndconv_oracle.c
 * (REAL = double / float, SFX = d / f).  TEST INFRASTRUCTURE ONLY.
 *
 * Restates what the reference gets from its FFT dependencies (rustfft 6.4,
 * realfft 3.5, called from src/conv_fft/processor/real.rs:40,62,84-98,183
 * and complex.rs:56,73): an unnormalised complex DFT in either direction, a
 * real-to-complex forward transform of length n returning n/2+1 bins, and
 * its complex-to-real inverse (unnormalised; the imaginary parts of the DC
 * and, for even n, Nyquist bins are ignored).
 *
 * Algorithm: iterative Stockham autosort over the prime factors of n with
 * specialised radix-2/4 butterflies and a generic O(p^2) butterfly for odd
 * primes up to ORC_GENERIC_MAXP; lengths with a larger prime factor go
 * through Bluestein's chirp-z transform with a power-of-two inner FFT.
 * Twiddles are evaluated in double and rounded once to REAL.
 */

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define CPLX CAT(cplx_, SFX)
#define PLAN CAT(fftplan_, SFX)
#define FN(name) CAT(name##_, SFX)

typedef struct { REAL re, im; } CPLX;

typedef struct PLAN {
    long n;
    int nst;            /* number of Stockham stages */
    int rad[64];        /* radix per stage */
    CPLX *tw;           /* tw[t] = exp(-2 pi i t / n), t < n */
    /* Bluestein */
    long m;             /* inner power-of-two length, 0 if unused */
    CPLX *chirp;        /* exp(-pi i k^2 / n), k < n */
    CPLX *bfk;          /* forward FFT (length m) of conj chirp, wrapped */
    struct PLAN *inner;
} PLAN;

static inline CPLX FN(cmul)(CPLX a, CPLX b) {
    CPLX r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}
static inline CPLX FN(cconj)(CPLX a) { CPLX r = {a.re, -a.im}; return r; }

static PLAN *FN(plan_create)(long n);
static void FN(orc_fft_exec)(const PLAN *p, const CPLX *in, CPLX *out, CPLX *scratch, int sign);

static void FN(plan_destroy)(PLAN *p) {
    if (!p) return;
    free(p->tw);
    free(p->chirp);
    free(p->bfk);
    FN(plan_destroy)(p->inner);
    free(p);
}

/* radix-r DFT of v in place, sign = -1 forward, +1 inverse */
static void FN(small_dft)(CPLX *v, int r, int sign, const PLAN *p) {
    if (r == 2) {
        CPLX a = v[0], b = v[1];
        v[0].re = a.re + b.re; v[0].im = a.im + b.im;
        v[1].re = a.re - b.re; v[1].im = a.im - b.im;
    } else if (r == 4) {
        CPLX a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3];
        CPLX s02 = {a0.re + a2.re, a0.im + a2.im}, d02 = {a0.re - a2.re, a0.im - a2.im};
        CPLX s13 = {a1.re + a3.re, a1.im + a3.im}, d13 = {a1.re - a3.re, a1.im - a3.im};
        /* multiply d13 by -i*sign... forward: W4 = -i */
        CPLX jd13;
        if (sign < 0) { jd13.re = d13.im; jd13.im = -d13.re; }   /* -i * d13 */
        else          { jd13.re = -d13.im; jd13.im = d13.re; }   /* +i * d13 */
        v[0].re = s02.re + s13.re; v[0].im = s02.im + s13.im;
        v[2].re = s02.re - s13.re; v[2].im = s02.im - s13.im;
        v[1].re = d02.re + jd13.re; v[1].im = d02.im + jd13.im;
        v[3].re = d02.re - jd13.re; v[3].im = d02.im - jd13.im;
    } else {
        /* generic DFT through the plan's twiddle table (n divisible by r) */
        CPLX out[ORC_GENERIC_MAXP];
        long step = p->n / r;
        for (int k = 0; k < r; k++) {
            REAL sre = 0, sim = 0;
            for (int j = 0; j < r; j++) {
                long e = ((long)j * k) % r * step;
                CPLX w = p->tw[e];
                if (sign > 0) w.im = -w.im;
                sre += v[j].re * w.re - v[j].im * w.im;
                sim += v[j].re * w.im + v[j].im * w.re;
            }
            out[k].re = sre; out[k].im = sim;
        }
        memcpy(v, out, sizeof(CPLX) * r);
    }
}

static PLAN *FN(plan_create)(long n) {
    PLAN *p = (PLAN *)calloc(1, sizeof(PLAN));
    p->n = n;
    long rem = n;
    int big = 0;
    /* radix order: 4s, 2, then odd primes ascending */
    while (rem % 4 == 0) { p->rad[p->nst++] = 4; rem /= 4; }
    while (rem % 2 == 0) { p->rad[p->nst++] = 2; rem /= 2; }
    for (long f = 3; f * f <= rem || rem > 1; f += 2) {
        if (f * f > rem) f = rem;
        while (rem % f == 0) {
            if (f > ORC_GENERIC_MAXP) big = 1;
            p->rad[p->nst++] = (int)f;
            rem /= f;
        }
        if (rem == 1) break;
    }
    p->tw = (CPLX *)malloc(sizeof(CPLX) * (n > 0 ? n : 1));
    for (long t = 0; t < n; t++) {
        double a = -2.0 * M_PI * (double)t / (double)n;
        p->tw[t].re = (REAL)cos(a);
        p->tw[t].im = (REAL)sin(a);
    }
    if (big) {
        long m = 1;
        while (m < 2 * n - 1) m <<= 1;
        p->m = m;
        p->chirp = (CPLX *)malloc(sizeof(CPLX) * n);
        for (long k = 0; k < n; k++) {
            long k2 = (long)(((unsigned long long)k * (unsigned long long)k) % (unsigned long long)(2 * n));
            double a = -M_PI * (double)k2 / (double)n;
            p->chirp[k].re = (REAL)cos(a);
            p->chirp[k].im = (REAL)sin(a);
        }
        p->inner = FN(plan_create)(m);
        CPLX *b = (CPLX *)calloc(m, sizeof(CPLX));
        for (long k = 0; k < n; k++) {
            b[k] = FN(cconj)(p->chirp[k]);
            if (k) b[m - k] = FN(cconj)(p->chirp[k]);
        }
        p->bfk = (CPLX *)malloc(sizeof(CPLX) * m);
        /* forward transform of b with the inner plan (no Bluestein there) */
        {
            CPLX *s = (CPLX *)malloc(sizeof(CPLX) * m);
            FN(orc_fft_exec)(p->inner, b, p->bfk, s, -1);
            free(s);
        }
        free(b);
    }
    return p;
}

/* out-of-place complex FFT; `in`, `out` and `scratch` must not overlap;
 * scratch holds max(n, 2m) elements (m = Bluestein inner length, else 0). */
static void FN(orc_fft_exec)(const PLAN *p, const CPLX *in, CPLX *out, CPLX *scratch, int sign) {
    long n = p->n;
    if (n == 1) { out[0] = in[0]; return; }
    if (p->m) {
        long m = p->m;
        CPLX *a = scratch, *fa = scratch + m;
        for (long k = 0; k < m; k++) { a[k].re = 0; a[k].im = 0; }
        for (long k = 0; k < n; k++) {
            CPLX c = p->chirp[k];
            if (sign > 0) c.im = -c.im;
            a[k] = FN(cmul)(in[k], c);
        }
        CPLX *s2 = (CPLX *)malloc(sizeof(CPLX) * m);
        FN(orc_fft_exec)(p->inner, a, fa, s2, -1);
        for (long k = 0; k < m; k++) {
            CPLX b = p->bfk[k];
            /* inverse direction uses conj chirp: FFT(conj(b)) with wrap is
               conj of FFT of b reversed; simpler: conj both sides */
            if (sign > 0) {
                /* spectrum of the conjugated filter: conj(B[(m-k)%m]) */
                b = FN(cconj)(p->bfk[(m - k) % m]);
            }
            fa[k] = FN(cmul)(fa[k], b);
        }
        FN(orc_fft_exec)(p->inner, fa, a, s2, +1);
        free(s2);
        for (long k = 0; k < n; k++) {
            CPLX c = p->chirp[k];
            if (sign > 0) c.im = -c.im;
            CPLX v = FN(cmul)(a[k], c);
            out[k].re = v.re / (REAL)m;
            out[k].im = v.im / (REAL)m;
        }
        return;
    }
    /* Stockham: ping-pong between out and scratch, ending in out */
    CPLX *src, *dst;
    int nst = p->nst;
    /* choose starting buffer so that the final stage writes into out */
    if (nst % 2 == 1) { dst = out; } else { dst = scratch; }
    src = (CPLX *)in;
    long Ns = 1;
    CPLX v[ORC_GENERIC_MAXP];
    for (int s = 0; s < nst; s++) {
        int R = p->rad[s];
        long nr = n / R;
        long twstep = n / (Ns * R);
        for (long j = 0; j < nr; j++) {
            long t = j % Ns;
            for (int r = 0; r < R; r++) {
                CPLX x = src[j + r * nr];
                if (r && t) {
                    CPLX w = p->tw[(t * r * twstep) % n];
                    if (sign > 0) w.im = -w.im;
                    x = FN(cmul)(x, w);
                }
                v[r] = x;
            }
            FN(small_dft)(v, R, sign, p);
            long base = (j / Ns) * Ns * R + t;
            for (int r = 0; r < R; r++) dst[base + r * Ns] = v[r];
        }
        Ns *= R;
        src = dst;
        dst = (dst == out) ? scratch : out;
    }
}

/* realfft-style forward: n reals -> n/2+1 complex bins */
static void FN(orc_rfft)(const PLAN *half, const PLAN *full, long n, const REAL *x,
                          CPLX *X, CPLX *work) {
    if (n % 2 == 0 && n >= 2) {
        long m = n / 2;
        CPLX *z = work, *Z = work + m, *s = work + 2 * m;
        for (long j = 0; j < m; j++) { z[j].re = x[2 * j]; z[j].im = x[2 * j + 1]; }
        FN(orc_fft_exec)(half, z, Z, s, -1);
        for (long k = 0; k <= m; k++) {
            CPLX a = Z[k % m], b = FN(cconj)(Z[(m - k) % m]);
            CPLX e = {(REAL)0.5 * (a.re + b.re), (REAL)0.5 * (a.im + b.im)};
            CPLX d = {(REAL)0.5 * (a.re - b.re), (REAL)0.5 * (a.im - b.im)};
            /* o = -i * d */
            CPLX o = {d.im, -d.re};
            double ang = -2.0 * M_PI * (double)k / (double)n;
            CPLX w = {(REAL)cos(ang), (REAL)sin(ang)};
            CPLX wo = FN(cmul)(w, o);
            X[k].re = e.re + wo.re;
            X[k].im = e.im + wo.im;
        }
    } else {
        CPLX *z = work, *Z = work + n, *s = work + 2 * n;
        for (long j = 0; j < n; j++) { z[j].re = x[j]; z[j].im = 0; }
        FN(orc_fft_exec)(full, z, Z, s, -1);
        for (long k = 0; k <= n / 2; k++) X[k] = Z[k];
    }
}

/* realfft-style inverse: n/2+1 bins -> n reals, unnormalised */
static void FN(orc_irfft)(const PLAN *half, const PLAN *full, long n, const CPLX *Xin,
                           REAL *x, CPLX *work) {
    if (n % 2 == 0 && n >= 2) {
        long m = n / 2;
        CPLX *Z = work, *z = work + m, *s = work + 2 * m;
        for (long k = 0; k < m; k++) {
            CPLX a = Xin[k], b = Xin[m - k];
            if (k == 0) { a.im = 0; b.im = 0; }
            b = FN(cconj)(b);
            CPLX e = {a.re + b.re, a.im + b.im};
            CPLX d = {a.re - b.re, a.im - b.im};
            double ang = 2.0 * M_PI * (double)k / (double)n;
            CPLX w = {(REAL)cos(ang), (REAL)sin(ang)};
            CPLX o = FN(cmul)(d, w);
            /* Z = e + i*o */
            Z[k].re = e.re - o.im;
            Z[k].im = e.im + o.re;
        }
        FN(orc_fft_exec)(half, Z, z, s, +1);
        for (long j = 0; j < m; j++) { x[2 * j] = z[j].re; x[2 * j + 1] = z[j].im; }
    } else {
        CPLX *Z = work, *z = work + n, *s = work + 2 * n;
        for (long k = 0; k <= n / 2; k++) {
            Z[k] = Xin[k];
            if (k == 0) Z[k].im = 0;
        }
        for (long k = n / 2 + 1; k < n; k++) Z[k] = FN(cconj)(Xin[n - k]);
        FN(orc_fft_exec)(full, Z, z, s, +1);
        for (long j = 0; j < n; j++) x[j] = z[j].re;
    }
}

/* scratch length (in CPLX) that is always enough for orc_rfft / orc_irfft /
 * orc_fft_exec on length n (any Bluestein inner length is < 4n) */
static long FN(work_len)(long n) {
    return 4 * n + 16 * n + 16;
}

#undef CPLX
#undef PLAN
#undef FN
