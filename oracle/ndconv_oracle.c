/*
 * ndconv oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference crate's convolution hot path
 * (ndarray-conv 0.6.1).  It is the oracle the CUDA library is tested
 * against and the timed CPU baseline; nothing in the product links or calls it.  Only
 * tests/, __graft_entry__.smoke() and bench.py (cpu baseline / reference
 * arm) load it.
 *
 * Every routine follows the reference's own sequence of steps so that its
 * results are the reference's results on the same inputs:
 *   - ConvMode::unfold                  src/conv/mod.rs:28-66
 *   - PaddingExt::padding / padding_in  src/padding/mod.rs:84-153,175-452,
 *                                       src/padding/dim.rs:34-157,
 *                                       src/padding/half_dim.rs:30-343
 *   - gen_offset_list                   src/dilation/mod.rs:34-60
 *   - ConvExt::conv                     src/conv/mod.rs:128-200
 *   - good_size                         src/conv_fft/good_size.rs:6-42
 *   - FFT buffers                       src/conv_fft/padding.rs:30-111
 *   - conv_fft_proc_impl                src/conv_fft/mod.rs:185-292
 *   - real / complex processors         src/conv_fft/processor/real.rs:105-281,
 *                                       src/conv_fft/processor/complex.rs:33-144
 * Where the reference panics (out-of-range reflect indices) the oracle
 * returns ORC_PAD_OUT_OF_RANGE.
 *
 * Parity pins: tests/test_oracle_golden.py re-asserts the reference's own
 * literal test vectors and the torch-computed fixtures in tests/golden/.
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#define ORC_GENERIC_MAXP 128

enum {
    ORC_OK = 0,
    ORC_DATA_SHAPE = 1,
    ORC_KERNEL_SHAPE = 2,
    ORC_MISMATCH_SHAPE = 3,
    ORC_PAD_OUT_OF_RANGE = 4,
    ORC_UNSUPPORTED = 5,
    ORC_INVALID = 6,
};
enum { DT_F32 = 0, DT_F64 = 1, DT_I32 = 2, DT_C32 = 3, DT_C64 = 4, DT_I64 = 5, DT_U8 = 6, DT_I8 = 7,
       DT_I16 = 8, DT_U16 = 9, DT_U32 = 10, DT_U64 = 11 };
enum { BT_ZEROS = 0, BT_CONST = 1, BT_REFLECT = 2, BT_REPLICATE = 3, BT_CIRCULAR = 4 };
enum { PM_ZEROS = 0, PM_CONST = 1, PM_REFLECT = 2, PM_REPLICATE = 3, PM_CIRCULAR = 4,
       PM_CUSTOM = 5, PM_EXPLICIT = 6 };
enum { CM_FULL = 0, CM_SAME = 1, CM_VALID = 2, CM_CUSTOM = 3, CM_EXPLICIT = 4 };

/* Problem description (same field layout as the library's descriptors so the
 * Python harness fills one structure for both). */
typedef struct {
    int32_t dtype, rank;
    int64_t xs[3];          /* data shape */
    int64_t ks[3];          /* kernel shape */
    int64_t dil[3];         /* dilation */
    int32_t reverse;        /* 1 = convolution (default), 0 = no_reverse */
    int32_t cmode;          /* ConvMode kind */
    int64_t cpad[3][2];     /* Custom: cpad[i][0]; Explicit: both */
    int64_t cstr[3];        /* Custom / Explicit strides */
    int32_t pmode;          /* PaddingMode kind */
    int32_t kinds[3][2];    /* Custom: kinds[i][0]; Explicit: per side */
    double vals[3][2][2];   /* BorderType::Const value (re, im) per side */
    double cval[2];         /* PaddingMode::Const value (re, im) */
} orc_problem;

/* ---------------------------------------------------------------- FFT --- */
#define REAL double
#define SFX d
#include "fft_impl.h"
#undef REAL
#undef SFX
#define REAL float
#define SFX f
#include "fft_impl.h"
#undef REAL
#undef SFX

/* ------------------------------------------------------- small helpers --- */
static long prod(const int64_t *s, int n) {
    long p = 1;
    for (int i = 0; i < n; i++) p *= (long)s[i];
    return p;
}
/* shape of rank <= 3 as three extents, leading axes filled with `fill` */
static void to3(const int64_t *shape, int rank, long fill, long *s3) {
    for (int i = 0; i < 3; i++) s3[i] = fill;
    for (int i = 0; i < rank; i++) s3[3 - rank + i] = (long)shape[i];
}
static void cstrides(const int64_t *shape, int rank, long *st) {
    long a = 1;
    for (int i = rank - 1; i >= 0; i--) { st[i] = a; a *= (long)shape[i]; }
}

/* good_size_cc, src/conv_fft/good_size.rs:6-31 (integer floor in /4*3, /6*5) */
long orc_good_size(long n) {
    long best = 1;
    while (best < n) best <<= 1;
    for (;;) {
        long nf = best / 4 * 3;
        if (nf < n) break;
        if (nf == n) return n;
        best = nf;
    }
    for (;;) {
        long nf = best / 6 * 5;
        if (nf < n) break;
        if (nf == n) return n;
        best = nf;
    }
    return best;
}

/* ConvMode::unfold, src/conv/mod.rs:28-66, on the dilated kernel extent
 * k + (k-1)(d-1) (src/conv/mod.rs:36-38). */
int orc_unfold(const orc_problem *p, int64_t pad[3][2], int64_t str[3]) {
    for (int i = 0; i < p->rank; i++) {
        int64_t ke = p->ks[i] * p->dil[i] - p->dil[i] + 1;
        switch (p->cmode) {
        case CM_FULL: pad[i][0] = pad[i][1] = ke - 1; str[i] = 1; break;
        case CM_SAME:
            if (ke % 2 == 0) { pad[i][0] = (ke - 1) / 2 + 1; pad[i][1] = (ke - 1) / 2; }
            else { pad[i][0] = pad[i][1] = (ke - 1) / 2; }
            str[i] = 1;
            break;
        case CM_VALID: pad[i][0] = pad[i][1] = 0; str[i] = 1; break;
        case CM_CUSTOM: pad[i][0] = pad[i][1] = p->cpad[i][0]; str[i] = p->cstr[i]; break;
        case CM_EXPLICIT: pad[i][0] = p->cpad[i][0]; pad[i][1] = p->cpad[i][1]; str[i] = p->cstr[i]; break;
        default: return ORC_INVALID;
        }
    }
    return ORC_OK;
}

/* ------------------------------------------------------------ padding --- */
/* Whole-hyperplane operations along `dim` of a buffer whose logical extents
 * are L and whose elements sit at the element strides of a possibly larger
 * allocation (the FFT-sized buffer of padding_in); an element is nc values
 * of vbytes bytes (8: double, 4: float).  These are ndarray's
 * index_axis_mut(Axis(dim), j).fill / .assign used by half_dim.rs.  Axes are
 * held in canonical three-axis form (leading extents 1). */
typedef struct {
    unsigned char *buf;
    int off;          /* 3 - rank: canonical index of axis 0 */
    long L[3];        /* logical extents */
    long st[3];       /* element strides of the allocation */
    int nc, vbytes;
} hbuf;

static void hb_init(hbuf *b, void *buf, int rank, const int64_t *L, const int64_t *alloc, int nc,
                    int vbytes) {
    long A[3];
    b->buf = (unsigned char *)buf;
    b->off = 3 - rank;
    to3(L, rank, 1, b->L);
    to3(alloc, rank, 1, A);
    b->st[2] = 1;
    b->st[1] = A[2];
    b->st[0] = A[1] * A[2];
    b->nc = nc;
    b->vbytes = vbytes;
}
static size_t hb_esz(const hbuf *b) { return (size_t)b->nc * (size_t)b->vbytes; }
static long hb_len(const hbuf *b, int dim) { return b->L[dim + b->off]; }
static unsigned char *hb_at(const hbuf *b, long i0, long i1, long i2) {
    return b->buf + (size_t)(i0 * b->st[0] + i1 * b->st[1] + i2 * b->st[2]) * hb_esz(b);
}

static void hp_fill(const hbuf *b, int dim, long j, const double *c) {
    unsigned char pat[16];
    for (int k = 0; k < b->nc; k++) {
        if (b->vbytes == 8) { double v = c[k]; memcpy(pat + 8 * k, &v, 8); }
        else { float v = (float)c[k]; memcpy(pat + 4 * k, &v, 4); }
    }
    const size_t esz = hb_esz(b);
    const int d = dim + b->off;
    long lo[3] = {0, 0, 0}, hi[3] = {b->L[0], b->L[1], b->L[2]};
    lo[d] = j;
    hi[d] = j + 1;
    for (long i0 = lo[0]; i0 < hi[0]; i0++)
        for (long i1 = lo[1]; i1 < hi[1]; i1++)
            for (long i2 = lo[2]; i2 < hi[2]; i2++) memcpy(hb_at(b, i0, i1, i2), pat, esz);
}
static void hp_copy(const hbuf *b, int dim, long dst, long src) {
    const size_t esz = hb_esz(b);
    const int d = dim + b->off;
    long hi[3] = {b->L[0], b->L[1], b->L[2]};
    hi[d] = 1;
    for (long i0 = 0; i0 < hi[0]; i0++)
        for (long i1 = 0; i1 < hi[1]; i1++) {
            if (d == 2) {
                memmove(hb_at(b, i0, i1, dst), hb_at(b, i0, i1, src), esz);
            } else {
                /* whole rows along the contiguous last axis */
                long a0 = i0, a1 = i1, s0 = i0, s1 = i1;
                if (d == 0) { a0 = dst; s0 = src; } else { a1 = dst; s1 = src; }
                memmove(hb_at(b, a0, a1, 0), hb_at(b, s0, s1, 0), esz * (size_t)b->L[2]);
            }
        }
}

/* half_dim.rs:30-343, one side of one axis; n = input extent on that axis */
static int half_front(const hbuf *b, int dim, long n, const int64_t pd[2], int kind, const double *c) {
    long L = hb_len(b, dim), p0 = pd[0];
    (void)n;
    switch (kind) {
    case BT_ZEROS: { double z[2] = {0, 0}; for (long j = 0; j < p0; j++) hp_fill(b, dim, j, z); break; }
    case BT_CONST: for (long j = 0; j < p0; j++) hp_fill(b, dim, j, c); break;
    case BT_REPLICATE: for (long j = 0; j < p0; j++) hp_copy(b, dim, j, p0); break;
    case BT_REFLECT:
        for (long j = 0; j < p0; j++) {
            long r = (p0 - j) + p0;
            if (r >= L) return ORC_PAD_OUT_OF_RANGE; /* index_axis panics */
            hp_copy(b, dim, j, r);
        }
        break;
    case BT_CIRCULAR:
        for (long j = 0; j < p0; j++) hp_copy(b, dim, j, L - pd[1] - (p0 - j));
        break;
    default: return ORC_INVALID;
    }
    return ORC_OK;
}
static int half_back(const hbuf *b, int dim, long n, const int64_t pd[2], int kind, const double *c) {
    long L = hb_len(b, dim), p0 = pd[0];
    long border = L - pd[1] - 1;
    switch (kind) {
    case BT_ZEROS: { double z[2] = {0, 0}; for (long j = n + p0; j < L; j++) hp_fill(b, dim, j, z); break; }
    case BT_CONST: for (long j = n + p0; j < L; j++) hp_fill(b, dim, j, c); break;
    case BT_REPLICATE: for (long j = n + p0; j < L; j++) hp_copy(b, dim, j, border); break;
    case BT_REFLECT:
        for (long j = n + p0; j < L; j++) {
            if (j - border > border) return ORC_PAD_OUT_OF_RANGE; /* usize underflow */
            hp_copy(b, dim, j, border - (j - border));
        }
        break;
    case BT_CIRCULAR:
        for (long j = n + p0; j < L; j++) hp_copy(b, dim, j, p0 + (j - border - 1));
        break;
    default: return ORC_INVALID;
    }
    return ORC_OK;
}

/* The per-axis border passes of PaddingExt::padding (fft_style = 0,
 * src/padding/mod.rs:84-117; Const was pre-filled) and padding_in
 * (fft_style = 1, mod.rs:119-153; Const filled per side), on a buffer that
 * already holds the input at [p0, p0 + n) on every axis: axes 0..rank-1 in
 * order, front side then back side. */
static int pad_passes(const orc_problem *p, const int64_t pad[3][2], const hbuf *b, int fft_style) {
    int st = ORC_OK;
    for (int d = 0; d < p->rank && st == ORC_OK; d++) {
        long n = p->xs[d];
        int kf, kb;
        const double *cf = NULL, *cb = NULL;
        switch (p->pmode) {
        case PM_ZEROS: continue;
        case PM_CONST:
            if (!fft_style) continue;           /* pre-filled instead */
            kf = kb = BT_CONST; cf = cb = p->cval; break;
        case PM_REFLECT: kf = kb = BT_REFLECT; break;
        case PM_REPLICATE: kf = kb = BT_REPLICATE; break;
        case PM_CIRCULAR: kf = kb = BT_CIRCULAR; break;
        case PM_CUSTOM: kf = kb = p->kinds[d][0]; cf = cb = p->vals[d][0]; break;
        case PM_EXPLICIT:
            kf = p->kinds[d][0]; kb = p->kinds[d][1]; cf = p->vals[d][0]; cb = p->vals[d][1];
            break;
        default: return ORC_INVALID;
        }
        st = half_front(b, d, n, pad[d], kf, cf);
        if (st == ORC_OK) st = half_back(b, d, n, pad[d], kb, cb);
    }
    return st;
}

/* PaddingExt::padding (fft_style = 0, src/padding/mod.rs:84-117) and
 * padding_in into a zeroed buffer (fft_style = 1, mod.rs:119-153).
 * x: contiguous, shape p->xs, nc doubles per element.
 * out: contiguous, shape xs[i] + pad[i][0] + pad[i][1]. */
int orc_padding(const orc_problem *p, const int64_t pad[3][2], const double *x, int nc,
                int fft_style, double *out) {
    int rank = p->rank;
    int64_t L[3];
    for (int i = 0; i < rank; i++) L[i] = p->xs[i] + pad[i][0] + pad[i][1];
    long total = prod(L, rank);
    double pre[2] = {0, 0};
    if (p->pmode == PM_CONST && !fft_style) { pre[0] = p->cval[0]; pre[1] = p->cval[1]; }
    for (long i = 0; i < total; i++)
        for (int c = 0; c < nc; c++) out[i * nc + c] = pre[c];
    /* padding_const: copy the input into [p0, p0+n) on every axis
     * (mod.rs:175-200), one contiguous last-axis row at a time */
    {
        long n3[3], L3[3], p3[3];
        to3(p->xs, rank, 1, n3);
        to3(L, rank, 1, L3);
        for (int i = 0; i < 3; i++) p3[i] = 0;
        for (int i = 0; i < rank; i++) p3[3 - rank + i] = pad[i][0];
        for (long i0 = 0; i0 < n3[0]; i0++)
            for (long i1 = 0; i1 < n3[1]; i1++)
                memcpy(out + (((i0 + p3[0]) * L3[1] + (i1 + p3[1])) * L3[2] + p3[2]) * nc,
                       x + ((i0 * n3[1] + i1) * n3[2]) * nc, sizeof(double) * (size_t)(n3[2] * nc));
    }
    hbuf b;
    hb_init(&b, out, rank, L, L, nc, (int)sizeof(double));
    return pad_passes(p, pad, &b, fft_style);
}

/* ------------------------------------------------------------ offsets --- */
/* gen_offset_list, src/dilation/mod.rs:34-60: iterate the (optionally
 * reversed) kernel in row-major order, drop exact zeros, offset =
 * sum idx[n] * dilation[n] * pds_stride[n].  k: nc doubles per element. */
long orc_taps(const orc_problem *p, const double *k, int nc, const long *pds_strides,
              long *offs, double *vals) {
    int rank = p->rank;
    long kst[3];
    cstrides(p->ks, rank, kst);
    long nk = prod(p->ks, rank), cnt = 0;
    for (long f = 0; f < nk; f++) {
        long r = f, src = 0, off = 0;
        for (int i = 0; i < rank; i++) {
            long idx = r / kst[i];
            r %= kst[i];
            long sidx = p->reverse ? (p->ks[i] - 1 - idx) : idx;
            src += sidx * kst[i];
            off += idx * p->dil[i] * pds_strides[i];
        }
        int zero = 1;
        for (int c = 0; c < nc; c++) if (k[src * nc + c] != 0.0) zero = 0;
        if (zero) continue;
        if (offs) offs[cnt] = off;
        if (vals) for (int c = 0; c < nc; c++) vals[cnt * nc + c] = k[src * nc + c];
        cnt++;
    }
    return cnt;
}

/* ---------------------------------------------------------- dtype io --- */
static int dt_nc(int dt) { return (dt == DT_C32 || dt == DT_C64) ? 2 : 1; }
static void to_double(int dt, const void *src, long n, double *dst) {
    long m = n * dt_nc(dt);
    switch (dt) {
    case DT_F32: case DT_C32: for (long i = 0; i < m; i++) dst[i] = ((const float *)src)[i]; break;
    case DT_F64: case DT_C64: memcpy(dst, src, sizeof(double) * m); break;
    case DT_I32: for (long i = 0; i < m; i++) dst[i] = ((const int32_t *)src)[i]; break;
    /* 64-bit values are exact while |v| <= 2^53 */
    case DT_I64: for (long i = 0; i < m; i++) dst[i] = (double)((const int64_t *)src)[i]; break;
    case DT_U64: for (long i = 0; i < m; i++) dst[i] = (double)((const uint64_t *)src)[i]; break;
    case DT_U8: for (long i = 0; i < m; i++) dst[i] = ((const uint8_t *)src)[i]; break;
    case DT_I8: for (long i = 0; i < m; i++) dst[i] = ((const int8_t *)src)[i]; break;
    case DT_I16: for (long i = 0; i < m; i++) dst[i] = ((const int16_t *)src)[i]; break;
    case DT_U16: for (long i = 0; i < m; i++) dst[i] = ((const uint16_t *)src)[i]; break;
    case DT_U32: for (long i = 0; i < m; i++) dst[i] = ((const uint32_t *)src)[i]; break;
    }
}

/* An integral double (|v| < 2^64) as the two's-complement bits of the
 * element: negative values through int64, the rest through uint64. */
static uint64_t int_bits(double v) { return v < 0 ? (uint64_t)(int64_t)v : (uint64_t)v; }

/* ------------------------------------------------------- direct conv --- */
static int shape_checks(const orc_problem *p, int kernel_code) {
    if (p->rank < 1 || p->rank > 3) return ORC_INVALID;
    if (prod(p->xs, p->rank) == 0) return ORC_DATA_SHAPE;
    if (prod(p->ks, p->rank) == 0) return kernel_code;
    for (int i = 0; i < p->rank; i++) if (p->dil[i] < 1) return ORC_INVALID;
    return ORC_OK;
}

/* ConvExt::conv, src/conv/mod.rs:128-200.  Accumulates in the element type
 * from zero, tap-list order (f32 in float, f64 in double, integers
 * wrapping as release-mode Rust: the sum of products modulo 2^64, then its
 * low 8 / 16 / 32 / 64 bits, which is the element type's own wrapping sum;
 * complex with the componentwise product of num-complex). ys receives the
 * output shape; y may be NULL to query it. */
int orc_conv(const orc_problem *p, const void *x, const void *k, int64_t *ys, void *y) {
    int st = shape_checks(p, ORC_KERNEL_SHAPE);
    if (st) return st;
    int rank = p->rank, dt = p->dtype, nc = dt_nc(dt);
    int64_t pad[3][2], str[3], L[3], ke[3];
    if ((st = orc_unfold(p, pad, str))) return st;
    for (int i = 0; i < rank; i++) {
        if (str[i] < 1) return ORC_INVALID;
        L[i] = p->xs[i] + pad[i][0] + pad[i][1];
        ke[i] = p->ks[i] * p->dil[i] - p->dil[i] + 1;
    }
    long nx = prod(p->xs, rank), nk = prod(p->ks, rank), nL = prod(L, rank);
    double *xd = malloc(sizeof(double) * nx * nc), *kd = malloc(sizeof(double) * nk * nc);
    double *pd = malloc(sizeof(double) * nL * nc);
    to_double(dt, x, nx, xd);
    to_double(dt, k, nk, kd);
    st = orc_padding(p, pad, xd, nc, 0, pd);
    if (st == ORC_OK)
        for (int i = 0; i < rank; i++) if (ke[i] > L[i]) st = ORC_MISMATCH_SHAPE;
    if (st) { free(xd); free(kd); free(pd); return st; }
    long pst[3];
    cstrides(L, rank, pst);
    long *offs = malloc(sizeof(long) * (nk + 1));
    double *tv = malloc(sizeof(double) * (nk + 1) * nc);
    long nt = orc_taps(p, kd, nc, pst, offs, tv);
    for (int i = 0; i < rank; i++) ys[i] = (pad[i][0] + pad[i][1] + p->xs[i] - ke[i]) / str[i] + 1;
    if (y) {
        long ny = prod(ys, rank), yst[3];
        cstrides(ys, rank, yst);
        for (long f = 0; f < ny; f++) {
            long r = f, anchor = 0;
            for (int i = 0; i < rank; i++) {
                long idx = r / yst[i];
                r %= yst[i];
                anchor += idx * str[i] * pst[i];
            }
            switch (dt) {
            case DT_F32: {
                float acc = 0.0f;
                for (long t = 0; t < nt; t++) acc += (float)pd[anchor + offs[t]] * (float)tv[t];
                ((float *)y)[f] = acc;
                break;
            }
            case DT_F64: {
                double acc = 0.0;
                for (long t = 0; t < nt; t++) acc += pd[anchor + offs[t]] * tv[t];
                ((double *)y)[f] = acc;
                break;
            }
            case DT_I32: case DT_I64: case DT_U8: case DT_I8: case DT_I16: case DT_U16: case DT_U32: case DT_U64: {
                uint64_t acc = 0;
                for (long t = 0; t < nt; t++) acc += int_bits(pd[anchor + offs[t]]) * int_bits(tv[t]);
                switch (dt) {
                case DT_U8: case DT_I8: ((uint8_t *)y)[f] = (uint8_t)acc; break;
                case DT_I16: case DT_U16: ((uint16_t *)y)[f] = (uint16_t)acc; break;
                case DT_I32: case DT_U32: ((uint32_t *)y)[f] = (uint32_t)acc; break;
                default: ((uint64_t *)y)[f] = acc; break;
                }
                break;
            }
            case DT_C32: {
                float ar = 0.0f, ai = 0.0f;
                for (long t = 0; t < nt; t++) {
                    float xr = (float)pd[2 * (anchor + offs[t])], xi = (float)pd[2 * (anchor + offs[t]) + 1];
                    float wr = (float)tv[2 * t], wi = (float)tv[2 * t + 1];
                    ar += xr * wr - xi * wi;
                    ai += xr * wi + xi * wr;
                }
                ((float *)y)[2 * f] = ar;
                ((float *)y)[2 * f + 1] = ai;
                break;
            }
            case DT_C64: {
                double ar = 0.0, ai = 0.0;
                for (long t = 0; t < nt; t++) {
                    double xr = pd[2 * (anchor + offs[t])], xi = pd[2 * (anchor + offs[t]) + 1];
                    double wr = tv[2 * t], wi = tv[2 * t + 1];
                    ar += xr * wr - xi * wi;
                    ai += xr * wi + xi * wr;
                }
                ((double *)y)[2 * f] = ar;
                ((double *)y)[2 * f + 1] = ai;
                break;
            }
            }
        }
    }
    free(xd); free(kd); free(pd); free(offs); free(tv);
    return ORC_OK;
}

/* ------------------------------------------------------ thread helper --- */
/* A fork-join parallel-for over [0, n) used where the reference uses rayon
 * (par_chunks_mut over rows, rayon::join, par_iter_mut). */
typedef void (*pf_fn)(void *ctx, long lo, long hi, int tid);
typedef struct { pf_fn fn; void *ctx; long lo, hi; int tid; } pf_job;
static void *pf_run(void *a) {
    pf_job *j = (pf_job *)a;
    if (j->lo < j->hi) j->fn(j->ctx, j->lo, j->hi, j->tid);
    return NULL;
}
/* grain: the fewest items worth a thread of their own, so that small
 * passes run on fewer threads (or inline) instead of paying for thread
 * start-up, as rayon's splitting does */
static int pf_count(long n, int nth, long grain) {
    if (grain < 1) grain = 1;
    if (nth > n / grain) nth = (int)(n / grain);
    return nth < 1 ? 1 : nth;
}
static void par_for(long n, int nth, long grain, pf_fn fn, void *ctx) {
    nth = pf_count(n, nth, grain);
    if (nth <= 1 || n < 2) { fn(ctx, 0, n, 0); return; }
    pthread_t th[256];
    pf_job jobs[256];
    if (nth > 256) nth = 256;
    for (int t = 0; t < nth; t++) {
        jobs[t].fn = fn; jobs[t].ctx = ctx; jobs[t].tid = t;
        jobs[t].lo = n * t / nth; jobs[t].hi = n * (t + 1) / nth;
    }
    for (int t = 1; t < nth; t++) pthread_create(&th[t], NULL, pf_run, &jobs[t]);
    pf_run(&jobs[0]);
    for (int t = 1; t < nth; t++) pthread_join(th[t], NULL);
}

/* --------------------------------------------- processor (per precision) --- */
#define REAL double
#define SFX d
#include "proc_impl.h"
#undef REAL
#undef SFX
#define REAL float
#define SFX f
#include "proc_impl.h"
#undef REAL
#undef SFX

/* ----------------------------------------------------- exported FFT API --- */
/* ConvFFTExt::conv_fft (nth = 1) / conv_fft_par (nth > 1) for f32, f64,
 * c32, c64 inputs (interleaved re/im for complex). */
int orc_conv_fft(const orc_problem *p, const void *x, const void *k, int64_t *ys, void *y, int nth) {
    switch (p->dtype) {
    case DT_F32: return conv_fft_f(p, 0, (const float *)x, (const float *)k, ys, (float *)y, nth);
    case DT_C32: return conv_fft_f(p, 1, (const float *)x, (const float *)k, ys, (float *)y, nth);
    case DT_F64: return conv_fft_d(p, 0, (const double *)x, (const double *)k, ys, (double *)y, nth);
    case DT_C64: return conv_fft_d(p, 1, (const double *)x, (const double *)k, ys, (double *)y, nth);
    default: return ORC_UNSUPPORTED;   /* integer FFT is documented broken upstream */
    }
}

/* Processor::forward for real (f32/f64) or complex (c32/c64) input of shape
 * s; out receives the spectrum in the processor's rotated layout and oshape
 * its shape.  Returns the remembered r2c length via *origin_len (real). */
int orc_fft_forward(int dtype, int rank, const int64_t *s, const void *in, void *out,
                    int64_t *oshape, int64_t *origin_len) {
    long n = prod(s, rank);
    *origin_len = s[rank - 1];
    switch (dtype) {
    case DT_F32: real_forward_f(rank, s, (const float *)in, (cplx_f *)out, oshape, 1); break;
    case DT_F64: real_forward_d(rank, s, (const double *)in, (cplx_d *)out, oshape, 1); break;
    case DT_C32: {
        cplx_f *tmp = malloc(sizeof(cplx_f) * n);
        memcpy(tmp, in, sizeof(cplx_f) * n);
        complex_transform_f(rank, s, tmp, (cplx_f *)out, oshape, 0, 1);
        free(tmp);
        break;
    }
    case DT_C64: {
        cplx_d *tmp = malloc(sizeof(cplx_d) * n);
        memcpy(tmp, in, sizeof(cplx_d) * n);
        complex_transform_d(rank, s, tmp, (cplx_d *)out, oshape, 0, 1);
        free(tmp);
        break;
    }
    default: return ORC_UNSUPPORTED;
    }
    return ORC_OK;
}

/* Processor::backward: spectrum of shape s (rotated layout) -> real array
 * (last axis origin_len) or complex array. */
int orc_fft_backward(int dtype, int rank, const int64_t *s, const void *in, int64_t origin_len,
                     void *out, int64_t *oshape) {
    long n = prod(s, rank);
    switch (dtype) {
    case DT_F32: case DT_C32: {
        cplx_f *tmp = malloc(sizeof(cplx_f) * n);
        memcpy(tmp, in, sizeof(cplx_f) * n);
        if (dtype == DT_F32) real_backward_f(rank, s, tmp, origin_len, (float *)out, oshape, 1);
        else complex_transform_f(rank, s, tmp, (cplx_f *)out, oshape, 1, 1);
        free(tmp);
        break;
    }
    case DT_F64: case DT_C64: {
        cplx_d *tmp = malloc(sizeof(cplx_d) * n);
        memcpy(tmp, in, sizeof(cplx_d) * n);
        if (dtype == DT_F64) real_backward_d(rank, s, tmp, origin_len, (double *)out, oshape, 1);
        else complex_transform_d(rank, s, tmp, (cplx_d *)out, oshape, 1, 1);
        free(tmp);
        break;
    }
    default: return ORC_UNSUPPORTED;
    }
    return ORC_OK;
}

/* Plain 1-D complex DFT of length n (sign -1 forward, +1 inverse,
 * unnormalised), f64, for checking the oracle's own FFT against numpy. */
void orc_fft1d(long n, const double *in, double *out, int sign) {
    fftplan_d *pl = plan_create_d(n);
    cplx_d *s = malloc(sizeof(cplx_d) * work_len_d(n));
    orc_fft_exec_d(pl, (const cplx_d *)in, (cplx_d *)out, s, sign);
    free(s);
    plan_destroy_d(pl);
}

/* padding::data / padding::kernel buffers (conv_fft/padding.rs:30-111) for
 * the golden tests; real doubles, fft_size given. */
int orc_fft_buffers(const orc_problem *p, const int64_t *fft_size, const double *x, const double *k,
                    double *dbuf, double *kbuf) {
    int rank = p->rank, st;
    int64_t pad[3][2], str[3], pds[3];
    if ((st = orc_unfold(p, pad, str))) return st;
    for (int i = 0; i < rank; i++) pds[i] = p->xs[i] + pad[i][0] + pad[i][1];
    long npd = prod(pds, rank), nF = prod(fft_size, rank), nk = prod(p->ks, rank);
    double *pd = malloc(sizeof(double) * npd);
    st = orc_padding(p, pad, x, 1, 1, pd);
    if (st) { free(pd); return st; }
    long pst[3], fst[3], kst[3];
    cstrides(pds, rank, pst);
    cstrides(fft_size, rank, fst);
    cstrides(p->ks, rank, kst);
    for (long i = 0; i < nF; i++) { dbuf[i] = 0; kbuf[i] = 0; }
    /* the data buffer is only defined when the padded data fits fft_size */
    int fits = 1;
    for (int i = 0; i < rank; i++) if (pds[i] > fft_size[i]) fits = 0;
    for (long f = 0; fits && f < npd; f++) {
        long r = f, o = 0;
        for (int i = 0; i < rank; i++) { long idx = r / pst[i]; r %= pst[i]; o += idx * fst[i]; }
        dbuf[o] = pd[f];
    }
    free(pd);
    for (long f = 0; f < nk; f++) {
        long r = f, o = 0;
        for (int i = 0; i < rank; i++) {
            long idx = r / kst[i];
            r %= kst[i];
            long ke = p->ks[i] * p->dil[i] - p->dil[i] + 1;
            o += (p->reverse ? idx * p->dil[i] : (ke - 1 - idx * p->dil[i])) * fst[i];
        }
        kbuf[o] = k[f];
    }
    return ORC_OK;
}
