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
 * Twiddles are evaluated in double and rounded once to REAL; the plan keeps
 * each stage's twiddles contiguously (tw[t*r*n/(Ns*R)] for t < Ns, 0 < r < R)
 * so the stage loops need no divisions.  This evaluates the same transform
 * as a textbook FFT at O(n log n) cost, so that the oracle, when timed as the
 * CPU baseline, is not slowed by the restatement itself.
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
    CPLX *stw;          /* stage twiddles: stage s at soff[s], [t][r-1] */
    long soff[64];
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
    free(p->stw);
    free(p->chirp);
    free(p->bfk);
    FN(plan_destroy)(p->inner);
    free(p);
}

/* radix-2 and radix-4 butterflies in place, sign = -1 forward, +1 inverse */
static inline void FN(bfly2)(CPLX *v) {
    CPLX a = v[0], b = v[1];
    v[0].re = a.re + b.re; v[0].im = a.im + b.im;
    v[1].re = a.re - b.re; v[1].im = a.im - b.im;
}
static inline void FN(bfly4)(CPLX *v, int sign) {
    CPLX a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3];
    CPLX s02 = {a0.re + a2.re, a0.im + a2.im}, d02 = {a0.re - a2.re, a0.im - a2.im};
    CPLX s13 = {a1.re + a3.re, a1.im + a3.im}, d13 = {a1.re - a3.re, a1.im - a3.im};
    CPLX jd13;  /* -i * d13 forward, +i * d13 inverse */
    if (sign < 0) { jd13.re = d13.im; jd13.im = -d13.re; }
    else          { jd13.re = -d13.im; jd13.im = d13.re; }
    v[0].re = s02.re + s13.re; v[0].im = s02.im + s13.im;
    v[2].re = s02.re - s13.re; v[2].im = s02.im - s13.im;
    v[1].re = d02.re + jd13.re; v[1].im = d02.im + jd13.im;
    v[3].re = d02.re - jd13.re; v[3].im = d02.im - jd13.im;
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
            long jk = 0;  /* (j * k) mod r, stepped */
            for (int j = 0; j < r; j++) {
                CPLX w = p->tw[jk * step];
                jk += k;
                if (jk >= r) jk -= r;
                if (sign > 0) w.im = -w.im;
                sre += v[j].re * w.re - v[j].im * w.im;
                sim += v[j].re * w.im + v[j].im * w.re;
            }
            out[k].re = sre; out[k].im = sim;
        }
        for (int k = 0; k < r; k++) v[k] = out[k];
    }
}

/* x times the stage twiddle w, conjugated when sign > 0 */
static inline CPLX FN(twmul)(CPLX x, CPLX w, int sign) {
    if (sign > 0) w.im = -w.im;
    return FN(cmul)(x, w);
}

/* One Stockham stage over the whole array: butterfly j = q * Ns + t
 * (q < nr / Ns, t < Ns) reads src[j + r * nr] and writes
 * dst[q * Ns * R + t + r * Ns]; input r > 0 of a butterfly with t > 0 is
 * multiplied by its twiddle W[t * (R - 1) + r - 1] (conjugated for
 * sign > 0). */
static void FN(stage2)(const CPLX *src, CPLX *dst, long nr, long Ns, const CPLX *W, int sign) {
    for (long q = 0; q < nr / Ns; q++) {
        const CPLX *in = src + q * Ns;
        CPLX *out = dst + q * Ns * 2;
        for (long t = 0; t < Ns; t++) {
            CPLX v[2] = {in[t], in[t + nr]};
            if (t) v[1] = FN(twmul)(v[1], W[t], sign);
            FN(bfly2)(v);
            out[t] = v[0];
            out[t + Ns] = v[1];
        }
    }
}
static void FN(stage4)(const CPLX *src, CPLX *dst, long nr, long Ns, const CPLX *W, int sign) {
    for (long q = 0; q < nr / Ns; q++) {
        const CPLX *in = src + q * Ns;
        CPLX *out = dst + q * Ns * 4;
        for (long t = 0; t < Ns; t++) {
            CPLX v[4] = {in[t], in[t + nr], in[t + 2 * nr], in[t + 3 * nr]};
            if (t) {
                const CPLX *w = W + t * 3;
                v[1] = FN(twmul)(v[1], w[0], sign);
                v[2] = FN(twmul)(v[2], w[1], sign);
                v[3] = FN(twmul)(v[3], w[2], sign);
            }
            FN(bfly4)(v, sign);
            out[t] = v[0];
            out[t + Ns] = v[1];
            out[t + 2 * Ns] = v[2];
            out[t + 3 * Ns] = v[3];
        }
    }
}

/* Length-R DFT of v for odd R, pairing inputs j and R - j:
 *   y[k]     = x0 + sum_j a_j cos(2 pi jk/R) -/+ i sum_j b_j sin(2 pi jk/R)
 *   y[R - k] = x0 + sum_j a_j cos(2 pi jk/R) +/- i sum_j b_j sin(2 pi jk/R)
 * with a_j = x_j + x_{R-j}, b_j = x_j - x_{R-j}, j, k = 1..(R-1)/2 (upper
 * signs forward).  cs[m] = cos(2 pi m/R), sn[m] = sin(2 pi m/R). */
static inline void FN(odd_dft)(CPLX *v, int R, int sign, const REAL *cs, const REAL *sn) {
    const int h = (R - 1) / 2;
    CPLX a[ORC_GENERIC_MAXP / 2], b[ORC_GENERIC_MAXP / 2];
    CPLX y0 = v[0];
    for (int j = 1; j <= h; j++) {
        a[j].re = v[j].re + v[R - j].re; a[j].im = v[j].im + v[R - j].im;
        b[j].re = v[j].re - v[R - j].re; b[j].im = v[j].im - v[R - j].im;
        y0.re += a[j].re; y0.im += a[j].im;
    }
    for (int k = 1; k <= h; k++) {
        REAL ar = v[0].re, ai = v[0].im, br = 0, bi = 0;
        int m = 0;
        for (int j = 1; j <= h; j++) {
            m += k;
            if (m >= R) m -= R;      /* m = j k mod R */
            ar += a[j].re * cs[m]; ai += a[j].im * cs[m];
            br += b[j].re * sn[m]; bi += b[j].im * sn[m];
        }
        if (sign < 0) {
            v[k].re = ar + bi; v[k].im = ai - br;
            v[R - k].re = ar - bi; v[R - k].im = ai + br;
        } else {
            v[k].re = ar - bi; v[k].im = ai + br;
            v[R - k].re = ar + bi; v[R - k].im = ai - br;
        }
    }
    v[0] = y0;
}

static void FN(stage_generic)(const CPLX *src, CPLX *dst, long nr, long Ns, int R, const CPLX *W,
                              int sign, const PLAN *p) {
    CPLX v[ORC_GENERIC_MAXP];
    REAL cs[ORC_GENERIC_MAXP], sn[ORC_GENERIC_MAXP];
    const int odd = R % 2 == 1;
    if (odd) {
        /* tw[m n / R] = exp(-2 pi i m / R) */
        const long step = p->n / R;
        for (int m = 0; m < R; m++) { cs[m] = p->tw[m * step].re; sn[m] = -p->tw[m * step].im; }
    }
    for (long q = 0; q < nr / Ns; q++) {
        const CPLX *in = src + q * Ns;
        CPLX *out = dst + q * Ns * R;
        for (long t = 0; t < Ns; t++) {
            for (int r = 0; r < R; r++) {
                CPLX x = in[t + r * nr];
                if (r && t) x = FN(twmul)(x, W[t * (R - 1) + (r - 1)], sign);
                v[r] = x;
            }
            if (odd) FN(odd_dft)(v, R, sign, cs, sn);
            else FN(small_dft)(v, R, sign, p);
            for (int r = 0; r < R; r++) out[t + r * Ns] = v[r];
        }
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
    {
        /* for n divisible by 4 only the first quarter is evaluated; the rest
         * follows exactly from tw[t + n/4] = -i tw[t] */
        const long q = n % 4 == 0 ? n / 4 : n;
        for (long t = 0; t < q; t++) {
            double a = -2.0 * M_PI * (double)t / (double)n;
            p->tw[t].re = (REAL)cos(a);
            p->tw[t].im = (REAL)sin(a);
        }
        for (long t = q; t < n; t++) {
            p->tw[t].re = p->tw[t - q].im;
            p->tw[t].im = -p->tw[t - q].re;
        }
    }
    {
        /* stage s (radix R, Ns = product of the earlier radices) multiplies
         * input r of butterfly t by tw[t * r * n / (Ns * R)], t * r < Ns * R */
        long tot = 0, Ns = 1;
        for (int st = 0; st < p->nst; st++) {
            p->soff[st] = tot;
            tot += Ns * (p->rad[st] - 1);
            Ns *= p->rad[st];
        }
        p->stw = (CPLX *)malloc(sizeof(CPLX) * (tot > 0 ? tot : 1));
        Ns = 1;
        for (int st = 0; st < p->nst; st++) {
            int R = p->rad[st];
            long step = n / (Ns * R);
            CPLX *w = p->stw + p->soff[st];
            for (long t = 0; t < Ns; t++)
                for (int r = 1; r < R; r++) w[t * (R - 1) + (r - 1)] = p->tw[t * r * step];
            Ns *= R;
        }
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
    for (int s = 0; s < nst; s++) {
        int R = p->rad[s];
        long nr = n / R;
        const CPLX *W = p->stw + p->soff[s];
        if (R == 4) FN(stage4)(src, dst, nr, Ns, W, sign);
        else if (R == 2) FN(stage2)(src, dst, nr, Ns, W, sign);
        else FN(stage_generic)(src, dst, nr, Ns, R, W, sign, p);
        Ns *= R;
        src = dst;
        dst = (dst == out) ? scratch : out;
    }
}

/* ------------------------------------------------- batched transforms ---
 * ORC_BATCH transforms of one plan at a time, stored element-major in split
 * form: x[(2 j) B + b] = Re x_b[j], x[(2 j + 1) B + b] = Im x_b[j], b < B.
 * Every stage runs the scalar path's butterflies with the same operation
 * order; the innermost loop runs over the B transforms, which the compiler
 * turns into SIMD code with portable flags.  Plans that need Bluestein
 * (a prime factor above ORC_GENERIC_MAXP) are not batched. */
#ifndef ORC_BATCH
#define ORC_BATCH 16
#endif

/* x[b] *= w (conjugated for sign > 0), over B split lanes */
static inline void FN(bt_twiddle)(REAL *xr, REAL *xi, CPLX w, int sign, int B) {
    const REAL wr = w.re, wi = sign > 0 ? -w.im : w.im;
    for (int b = 0; b < B; b++) {
        const REAL r = xr[b] * wr - xi[b] * wi, i = xr[b] * wi + xi[b] * wr;
        xr[b] = r;
        xi[b] = i;
    }
}

/* Result in x; scratch holds 2 n B REALs. */
static void FN(fft_batch)(const PLAN *p, REAL *x, REAL *scratch, int B, int sign) {
    const long n = p->n;
    if (n == 1) return;
    REAL *src = x, *dst = scratch;
    long Ns = 1;
    const REAL sg = sign < 0 ? (REAL)1 : (REAL)-1;  /* W4 = -i forward, +i inverse */
    REAL vr[ORC_GENERIC_MAXP][ORC_BATCH], vi[ORC_GENERIC_MAXP][ORC_BATCH];
    for (int s = 0; s < p->nst; s++) {
        const int R = p->rad[s];
        const long nr = n / R;
        const CPLX *W = p->stw + p->soff[s];
        REAL cs[ORC_GENERIC_MAXP], sn[ORC_GENERIC_MAXP];
        if (R != 2 && R != 4) {
            const long step = n / R;
            for (int m = 0; m < R; m++) { cs[m] = p->tw[m * step].re; sn[m] = -p->tw[m * step].im; }
        }
        for (long q = 0; q < nr / Ns; q++)
            for (long t = 0; t < Ns; t++) {
                const long j = q * Ns + t, base = q * Ns * R + t;
                /* gather the R inputs (twiddled) into vr / vi */
                for (int r = 0; r < R; r++) {
                    const REAL *ir = src + 2 * (j + r * nr) * B, *ii = ir + B;
                    for (int b = 0; b < B; b++) { vr[r][b] = ir[b]; vi[r][b] = ii[b]; }
                    if (r && t) FN(bt_twiddle)(vr[r], vi[r], W[t * (R - 1) + (r - 1)], sign, B);
                }
                if (R == 2) {
                    for (int b = 0; b < B; b++) {
                        const REAL ar = vr[0][b], ai = vi[0][b], br = vr[1][b], bi = vi[1][b];
                        vr[0][b] = ar + br; vi[0][b] = ai + bi;
                        vr[1][b] = ar - br; vi[1][b] = ai - bi;
                    }
                } else if (R == 4) {
                    for (int b = 0; b < B; b++) {
                        const REAL s02r = vr[0][b] + vr[2][b], s02i = vi[0][b] + vi[2][b];
                        const REAL d02r = vr[0][b] - vr[2][b], d02i = vi[0][b] - vi[2][b];
                        const REAL s13r = vr[1][b] + vr[3][b], s13i = vi[1][b] + vi[3][b];
                        const REAL d13r = vr[1][b] - vr[3][b], d13i = vi[1][b] - vi[3][b];
                        const REAL jr = sg * d13i, ji = -sg * d13r;
                        vr[0][b] = s02r + s13r; vi[0][b] = s02i + s13i;
                        vr[2][b] = s02r - s13r; vi[2][b] = s02i - s13i;
                        vr[1][b] = d02r + jr; vi[1][b] = d02i + ji;
                        vr[3][b] = d02r - jr; vi[3][b] = d02i - ji;
                    }
                } else {
                    /* odd R: the paired form of odd_dft, lane by lane */
                    const int h = (R - 1) / 2;
                    REAL ar[ORC_BATCH], ai[ORC_BATCH], br[ORC_BATCH], bi[ORC_BATCH];
                    REAL y0r[ORC_BATCH], y0i[ORC_BATCH];
                    for (int b = 0; b < B; b++) { y0r[b] = vr[0][b]; y0i[b] = vi[0][b]; }
                    for (int jj = 1; jj <= h; jj++)
                        for (int b = 0; b < B; b++) {
                            const REAL pr = vr[jj][b] + vr[R - jj][b], pi = vi[jj][b] + vi[R - jj][b];
                            const REAL mr = vr[jj][b] - vr[R - jj][b], mi = vi[jj][b] - vi[R - jj][b];
                            vr[jj][b] = pr; vi[jj][b] = pi;          /* a_j */
                            vr[R - jj][b] = mr; vi[R - jj][b] = mi;  /* b_j */
                            y0r[b] += pr; y0i[b] += pi;
                        }
                    REAL outr[ORC_GENERIC_MAXP][ORC_BATCH], outi[ORC_GENERIC_MAXP][ORC_BATCH];
                    for (int k = 1; k <= h; k++) {
                        for (int b = 0; b < B; b++) { ar[b] = vr[0][b]; ai[b] = vi[0][b]; br[b] = 0; bi[b] = 0; }
                        int m = 0;
                        for (int jj = 1; jj <= h; jj++) {
                            m += k;
                            if (m >= R) m -= R;
                            const REAL c = cs[m], sv = sn[m];
                            for (int b = 0; b < B; b++) {
                                ar[b] += vr[jj][b] * c; ai[b] += vi[jj][b] * c;
                                br[b] += vr[R - jj][b] * sv; bi[b] += vi[R - jj][b] * sv;
                            }
                        }
                        for (int b = 0; b < B; b++) {
                            if (sign < 0) {
                                outr[k][b] = ar[b] + bi[b]; outi[k][b] = ai[b] - br[b];
                                outr[R - k][b] = ar[b] - bi[b]; outi[R - k][b] = ai[b] + br[b];
                            } else {
                                outr[k][b] = ar[b] - bi[b]; outi[k][b] = ai[b] + br[b];
                                outr[R - k][b] = ar[b] + bi[b]; outi[R - k][b] = ai[b] - br[b];
                            }
                        }
                    }
                    for (int b = 0; b < B; b++) { vr[0][b] = y0r[b]; vi[0][b] = y0i[b]; }
                    for (int r = 1; r < R; r++)
                        for (int b = 0; b < B; b++) { vr[r][b] = outr[r][b]; vi[r][b] = outi[r][b]; }
                }
                for (int r = 0; r < R; r++) {
                    REAL *orr = dst + 2 * (base + r * Ns) * B, *oi = orr + B;
                    for (int b = 0; b < B; b++) { orr[b] = vr[r][b]; oi[b] = vi[r][b]; }
                }
            }
        Ns *= R;
        REAL *tmp = src;
        src = dst;
        dst = tmp;
    }
    if (src != x) memcpy(x, src, sizeof(REAL) * 2 * (size_t)n * (size_t)B);
}

/* realfft-style forward for even n, last step: the half-length transform
 * Z (m = n/2 bins at Zr[k * zs], Zi[k * zs]) of z[j] = x[2j] + i x[2j+1]
 * gives the n/2+1 bins X[k] = E[k] + exp(-2 pi i k/n) (-i) D[k], with
 * E, D the even / odd halves 0.5 (Z[k] +- conj Z[m-k]). */
static void FN(rfft_post)(const PLAN *full, long n, const REAL *Zr, const REAL *Zi, long zs, CPLX *X) {
    const long m = n / 2;
    for (long k = 0; k <= m; k++) {
        const long ka = k % m, kb = (m - k) % m;
        CPLX a = {Zr[ka * zs], Zi[ka * zs]}, b = {Zr[kb * zs], -Zi[kb * zs]};
        CPLX e = {(REAL)0.5 * (a.re + b.re), (REAL)0.5 * (a.im + b.im)};
        CPLX d = {(REAL)0.5 * (a.re - b.re), (REAL)0.5 * (a.im - b.im)};
        /* o = -i * d */
        CPLX o = {d.im, -d.re};
        CPLX w = full->tw[k];  /* exp(-2 pi i k / n) */
        CPLX wo = FN(cmul)(w, o);
        X[k].re = e.re + wo.re;
        X[k].im = e.im + wo.im;
    }
}

/* realfft-style inverse for even n, first step: the half-length spectrum
 * Z[k] = E[k] + i exp(+2 pi i k/n) D[k] (written to Zr / Zi with stride
 * zs), whose unnormalised inverse transform interleaves the n reals. */
static void FN(irfft_pre)(const PLAN *full, long n, const CPLX *Xin, REAL *Zr, REAL *Zi, long zs) {
    const long m = n / 2;
    for (long k = 0; k < m; k++) {
        CPLX a = Xin[k], b = Xin[m - k];
        if (k == 0) { a.im = 0; b.im = 0; }
        b = FN(cconj)(b);
        CPLX e = {a.re + b.re, a.im + b.im};
        CPLX d = {a.re - b.re, a.im - b.im};
        CPLX w = FN(cconj)(full->tw[k]);  /* exp(+2 pi i k / n) */
        CPLX o = FN(cmul)(d, w);
        /* Z = e + i*o */
        Zr[k * zs] = e.re - o.im;
        Zi[k * zs] = e.im + o.re;
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
        FN(rfft_post)(full, n, &Z[0].re, &Z[0].im, 2, X);
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
        FN(irfft_pre)(full, n, Xin, &Z[0].re, &Z[0].im, 2);
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
 * orc_fft_exec on length n (any Bluestein inner length is < 4n), or for
 * ORC_BATCH batched transforms of length n (two split buffers) */
static long FN(work_len)(long n) {
    return 4 * n + 16 * n + 16 + 2 * (long)ORC_BATCH * n;  /* + batched buffers */
}

#undef CPLX
#undef PLAN
#undef FN
