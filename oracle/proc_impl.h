/*
 * Oracle FFT processors and FFT convolution, instantiated per precision by
 * ndconv_oracle.c (REAL = double / float).  TEST INFRASTRUCTURE ONLY.
 *
 * Layout and steps follow src/conv_fft/processor/real.rs:105-281 and
 * src/conv_fft/processor/complex.rs:33-144:
 *   real forward : r2c on the last axis, then N-1 x (rotate axes right,
 *                  contiguous copy, c2c forward on the new last axis)
 *   real backward: N-1 x (c2c inverse on the last axis, rotate axes left,
 *                  copy), c2r of the remembered length, divide by the count
 *   complex      : N c2c passes with a rotation between consecutive passes;
 *                  backward divides by the element count.
 * Rotating a contiguous N-d array right (last axis to the front) is the
 * transpose of its [prod(others)] x [last] matrix; rotating left is the
 * transpose of [first] x [prod(others)].
 */

#define CPLX CAT(cplx_, SFX)
#define PLAN CAT(fftplan_, SFX)
#define FN(name) CAT(name##_, SFX)

static void FN(transpose)(const CPLX *a, CPLX *b, long rows, long cols) {
    /* b[c][r] = a[r][c], blocked */
    const long B = 32;
    for (long r0 = 0; r0 < rows; r0 += B)
        for (long c0 = 0; c0 < cols; c0 += B) {
            long r1 = r0 + B < rows ? r0 + B : rows, c1 = c0 + B < cols ? c0 + B : cols;
            for (long r = r0; r < r1; r++)
                for (long c = c0; c < c1; c++) b[c * rows + r] = a[r * cols + c];
        }
}

typedef struct {
    const PLAN *plan;
    const CPLX *in;
    CPLX *out;
    long len;
    int sign;
    CPLX **work;
} FN(rows_ctx);

/* Rows [lo, hi) in blocks of ORC_BATCH through the batched transform (rows
 * gathered into the split element-major layout and scattered back); plans
 * with a Bluestein stage, and fewer than four rows, go row by row. */
static void FN(rows_c2c_worker)(void *vc, long lo, long hi, int tid) {
    FN(rows_ctx) *c = (FN(rows_ctx) *)vc;
    const long len = c->len;
    if (c->plan->m || len < 2 || hi - lo < 4) {
        for (long r = lo; r < hi; r++)
            FN(orc_fft_exec)(c->plan, c->in + r * len, c->out + r * len, c->work[tid], c->sign);
        return;
    }
    REAL *xb = (REAL *)c->work[tid], *sb = xb + 2 * len * ORC_BATCH;
    for (long r0 = lo; r0 < hi; r0 += ORC_BATCH) {
        const int B = (int)(hi - r0 < ORC_BATCH ? hi - r0 : ORC_BATCH);
        const CPLX *in = c->in + r0 * len;
        for (long j = 0; j < len; j++)
            for (int b = 0; b < B; b++) {
                xb[2 * j * B + b] = in[b * len + j].re;
                xb[(2 * j + 1) * B + b] = in[b * len + j].im;
            }
        FN(fft_batch)(c->plan, xb, sb, B, c->sign);
        CPLX *out = c->out + r0 * len;
        for (long j = 0; j < len; j++)
            for (int b = 0; b < B; b++) {
                out[b * len + j].re = xb[2 * j * B + b];
                out[b * len + j].im = xb[(2 * j + 1) * B + b];
            }
    }
}

/* rows per thread at least: ~32k samples of work, and four rows so that
 * the batched transforms apply */
static long FN(row_grain)(long len) {
    long g = 32768 / (len > 0 ? len : 1);
    return g < 4 ? 4 : g;
}

static CPLX **FN(alloc_work)(int nth, long n) {
    CPLX **w = (CPLX **)malloc(sizeof(CPLX *) * nth);
    for (int t = 0; t < nth; t++) w[t] = (CPLX *)malloc(sizeof(CPLX) * FN(work_len)(n));
    return w;
}
static void FN(free_work)(CPLX **w, int nth) {
    for (int t = 0; t < nth; t++) free(w[t]);
    free(w);
}

/* c2c along the last axis of a [rows][len] array (out-of-place) */
static void FN(rows_c2c)(const CPLX *in, CPLX *out, long rows, long len, int sign, int nth) {
    PLAN *pl = FN(plan_create)(len);
    int nt = pf_count(rows, nth < 1 ? 1 : nth, FN(row_grain)(len));
    CPLX **w = FN(alloc_work)(nt, len);
    FN(rows_ctx) c = {pl, in, out, len, sign, w};
    par_for(rows, nt, FN(row_grain)(len), FN(rows_c2c_worker), &c);
    FN(free_work)(w, nt);
    FN(plan_destroy)(pl);
}

typedef struct {
    const PLAN *half, *full;
    long n, h;
    const REAL *rin;
    CPLX *cin;
    REAL *rout;
    CPLX *cout;
    CPLX **work;
} FN(real_ctx);

/* Even-length rows go through the batched half-length transform in blocks
 * of ORC_BATCH rows; odd lengths, Bluestein plans and fewer than four rows
 * go row by row. */
static int FN(real_batched)(const FN(real_ctx) *c, long rows) {
    return c->n % 2 == 0 && c->n >= 4 && !c->half->m && rows >= 4;
}
static void FN(r2c_worker)(void *vc, long lo, long hi, int tid) {
    FN(real_ctx) *c = (FN(real_ctx) *)vc;
    const long n = c->n, m = n / 2;
    if (!FN(real_batched)(c, hi - lo)) {
        for (long r = lo; r < hi; r++)
            FN(orc_rfft)(c->half, c->full, n, c->rin + r * n, c->cout + r * c->h, c->work[tid]);
        return;
    }
    REAL *zb = (REAL *)c->work[tid], *sb = zb + 2 * m * ORC_BATCH;
    for (long r0 = lo; r0 < hi; r0 += ORC_BATCH) {
        const int B = (int)(hi - r0 < ORC_BATCH ? hi - r0 : ORC_BATCH);
        const REAL *x = c->rin + r0 * n;
        for (long j = 0; j < m; j++)
            for (int b = 0; b < B; b++) {
                zb[2 * j * B + b] = x[b * n + 2 * j];
                zb[(2 * j + 1) * B + b] = x[b * n + 2 * j + 1];
            }
        FN(fft_batch)(c->half, zb, sb, B, -1);
        for (int b = 0; b < B; b++)
            FN(rfft_post)(c->full, n, zb + b, zb + B + b, 2 * B, c->cout + (r0 + b) * c->h);
    }
}
static void FN(c2r_worker)(void *vc, long lo, long hi, int tid) {
    FN(real_ctx) *c = (FN(real_ctx) *)vc;
    const long n = c->n, m = n / 2;
    if (!FN(real_batched)(c, hi - lo)) {
        for (long r = lo; r < hi; r++)
            FN(orc_irfft)(c->half, c->full, n, c->cin + r * c->h, c->rout + r * n, c->work[tid]);
        return;
    }
    REAL *zb = (REAL *)c->work[tid], *sb = zb + 2 * m * ORC_BATCH;
    for (long r0 = lo; r0 < hi; r0 += ORC_BATCH) {
        const int B = (int)(hi - r0 < ORC_BATCH ? hi - r0 : ORC_BATCH);
        for (int b = 0; b < B; b++)
            FN(irfft_pre)(c->full, n, c->cin + (r0 + b) * c->h, zb + b, zb + B + b, 2 * B);
        FN(fft_batch)(c->half, zb, sb, B, +1);
        REAL *x = c->rout + r0 * n;
        for (long j = 0; j < m; j++)
            for (int b = 0; b < B; b++) {
                x[b * n + 2 * j] = zb[2 * j * B + b];
                x[b * n + 2 * j + 1] = zb[(2 * j + 1) * B + b];
            }
    }
}

/* real::Processor::forward: in shape s -> out (caller allocates prod with
 * last = n/2+1); oshape receives the rotated output shape. */
static void FN(real_forward)(int rank, const int64_t *s, const REAL *in, CPLX *out,
                             int64_t *oshape, int nth) {
    long n = s[rank - 1], h = n / 2 + 1;
    long rows = prod(s, rank - 1);
    int nt = pf_count(rows, nth < 1 ? 1 : nth, FN(row_grain)(n));
    PLAN *half = FN(plan_create)(n / 2 > 0 ? n / 2 : 1), *full = FN(plan_create)(n);
    CPLX **w = FN(alloc_work)(nt, n);
    FN(real_ctx) c = {half, full, n, h, in, NULL, NULL, out, w};
    par_for(rows, nt, FN(row_grain)(n), FN(r2c_worker), &c);
    FN(free_work)(w, nt);
    FN(plan_destroy)(half);
    FN(plan_destroy)(full);
    int64_t a[3];
    for (int i = 0; i < rank; i++) a[i] = s[i];
    a[rank - 1] = h;
    long tot = prod(a, rank);
    CPLX *buf = (CPLX *)malloc(sizeof(CPLX) * (tot ? tot : 1));
    for (int it = 0; it < rank - 1; it++) {
        long last = a[rank - 1], M = tot / last;
        FN(transpose)(out, buf, M, last);            /* rotate right */
        int64_t b[3];
        b[0] = a[rank - 1];
        for (int i = 1; i < rank; i++) b[i] = a[i - 1];
        memcpy(a, b, sizeof(b));
        FN(rows_c2c)(buf, out, tot / a[rank - 1], a[rank - 1], -1, nth);
    }
    free(buf);
    for (int i = 0; i < rank; i++) oshape[i] = a[i];
}

/* real::Processor::backward: in (complex, shape s) is consumed as scratch;
 * origin_len is the last forward's last-axis length. */
static void FN(real_backward)(int rank, const int64_t *s, CPLX *in, long origin_len, REAL *out,
                              int64_t *oshape, int nth) {
    int64_t a[3] = {1, 1, 1};
    for (int i = 0; i < rank; i++) a[i] = s[i];
    long tot = prod(a, rank);
    CPLX *buf = (CPLX *)malloc(sizeof(CPLX) * (tot ? tot : 1));
    for (int it = 0; it < rank - 1; it++) {
        FN(rows_c2c)(in, buf, tot / a[rank - 1], a[rank - 1], +1, nth);
        long first = a[0], M = tot / first;
        FN(transpose)(buf, in, first, M);            /* rotate left */
        int64_t b[3];
        for (int i = 0; i < rank - 1; i++) b[i] = a[i + 1];
        b[rank - 1] = a[0];
        memcpy(a, b, sizeof(b));
    }
    free(buf);
    long h = a[rank - 1], n = origin_len;
    long rows = tot / h;
    int nt = pf_count(rows, nth < 1 ? 1 : nth, FN(row_grain)(n));
    PLAN *half = FN(plan_create)(n / 2 > 0 ? n / 2 : 1), *full = FN(plan_create)(n);
    CPLX **w = FN(alloc_work)(nt, n);
    FN(real_ctx) c = {half, full, n, h, NULL, in, out, NULL, w};
    par_for(rows, nt, FN(row_grain)(n), FN(c2r_worker), &c);
    FN(free_work)(w, nt);
    FN(plan_destroy)(half);
    FN(plan_destroy)(full);
    a[rank - 1] = n;
    long count = prod(a, rank);
    REAL len = (REAL)count;
    for (long i = 0; i < count; i++) out[i] = out[i] / len;
    for (int i = 0; i < rank; i++) oshape[i] = a[i];
}

/* complex::Processor::internal (+ backward's division), complex.rs:33-144.
 * data is consumed as scratch; the result is written to out. */
static void FN(complex_transform)(int rank, const int64_t *s, CPLX *data, CPLX *out,
                                  int64_t *oshape, int inverse, int nth) {
    int64_t a[3];
    for (int i = 0; i < rank; i++) a[i] = s[i];
    long tot = prod(a, rank);
    for (int it = 0; it < rank; it++) {
        FN(rows_c2c)(data, out, tot / a[rank - 1], a[rank - 1], inverse ? +1 : -1, nth);
        if (it != rank - 1) {
            int64_t b[3];
            if (!inverse) {
                long last = a[rank - 1];
                FN(transpose)(out, data, tot / last, last);
                b[0] = a[rank - 1];
                for (int i = 1; i < rank; i++) b[i] = a[i - 1];
            } else {
                long first = a[0];
                FN(transpose)(out, data, first, tot / first);
                for (int i = 0; i < rank - 1; i++) b[i] = a[i + 1];
                b[rank - 1] = a[0];
            }
            memcpy(a, b, sizeof(b));
        }
    }
    if (inverse) {
        REAL len = (REAL)tot;
        for (long i = 0; i < tot; i++) { out[i].re = out[i].re / len; out[i].im = out[i].im / len; }
    }
    for (int i = 0; i < rank; i++) oshape[i] = a[i];
}

typedef struct { CPLX *d; const CPLX *k; } FN(mul_ctx);
static void FN(mul_worker)(void *vc, long lo, long hi, int tid) {
    (void)tid;
    FN(mul_ctx) *c = (FN(mul_ctx) *)vc;
    for (long i = lo; i < hi; i++) c->d[i] = FN(cmul)(c->d[i], c->k[i]);
}

/* conv_fft_proc_impl, src/conv_fft/mod.rs:185-292.  is_complex selects the
 * complex processor; x, k, y hold REAL (or interleaved re/im) values.
 * nth > 1 mirrors conv_fft_par's rayon decomposition (row-parallel passes,
 * parallel spectrum multiply); nth == 1 is conv_fft. */
static int FN(conv_fft)(const orc_problem *p, int is_complex, const REAL *x, const REAL *k,
                        int64_t *ys, REAL *y, int nth) {
    int st = shape_checks(p, ORC_DATA_SHAPE);   /* zero kernel -> DataShape (mod.rs:211-212) */
    if (st) return st;
    int rank = p->rank, nc = is_complex ? 2 : 1;
    int64_t pad[3][2], str[3], pds[3], ke[3], F[3];
    if ((st = orc_unfold(p, pad, str))) return st;
    for (int i = 0; i < rank; i++) {
        if (str[i] < 1) return ORC_INVALID;
        ke[i] = p->ks[i] * p->dil[i] - p->dil[i] + 1;
        pds[i] = p->xs[i] + pad[i][0] + pad[i][1];
        if (ke[i] > pds[i]) return ORC_MISMATCH_SHAPE;
    }
    for (int i = 0; i < rank; i++) F[i] = orc_good_size(pds[i] > ke[i] ? pds[i] : ke[i]);
    for (int i = 0; i < rank; i++) ys[i] = (pds[i] - ke[i]) / str[i] + 1;
    if (!y) return ORC_OK;

    long nx = prod(p->xs, rank), nk = prod(p->ks, rank), npd = prod(pds, rank), nF = prod(F, rank);
    REAL *dbuf = calloc(nF * nc, sizeof(REAL)), *kbuf = calloc(nF * nc, sizeof(REAL));
    /* canonical three-axis forms (leading extents 1) for the row loops below */
    long X3[3], F3[3], K3[3], D3[3], E3[3], Q3[3] = {0, 0, 0};
    to3(p->xs, rank, 1, X3);
    to3(F, rank, 1, F3);
    to3(p->ks, rank, 1, K3);
    to3(p->dil, rank, 1, D3);
    to3(ke, rank, 1, E3);
    for (int i = 0; i < rank; i++) Q3[3 - rank + i] = pad[i][0];
    (void)npd;
    (void)nx;
    /* padding::data (conv_fft/padding.rs:30-62): padding_in on the [0, pds)
     * box of the zeroed FFT buffer: the input at [p0, p0 + n) on every axis,
     * then the border passes axis by axis */
    for (long i0 = 0; i0 < X3[0]; i0++)
        for (long i1 = 0; i1 < X3[1]; i1++)
            memcpy(dbuf + (((i0 + Q3[0]) * F3[1] + (i1 + Q3[1])) * F3[2] + Q3[2]) * nc,
                   x + ((i0 * X3[1] + i1) * X3[2]) * nc, sizeof(REAL) * (size_t)(X3[2] * nc));
    {
        hbuf b;
        hb_init(&b, dbuf, rank, pds, F, nc, (int)sizeof(REAL));
        if ((st = pad_passes(p, pad, &b, 1))) {
            free(dbuf);
            free(kbuf);
            return st;
        }
    }
    /* padding::kernel (conv_fft/padding.rs:78-111): buf[i*d] = k[i], or at
     * k_eff-1-i*d (negative slice step) when !reverse */
    (void)nk;
    for (long i0 = 0; i0 < K3[0]; i0++)
        for (long i1 = 0; i1 < K3[1]; i1++)
            for (long i2 = 0; i2 < K3[2]; i2++) {
                long q0 = p->reverse ? i0 * D3[0] : E3[0] - 1 - i0 * D3[0];
                long q1 = p->reverse ? i1 * D3[1] : E3[1] - 1 - i1 * D3[1];
                long q2 = p->reverse ? i2 * D3[2] : E3[2] - 1 - i2 * D3[2];
                long o = (q0 * F3[1] + q1) * F3[2] + q2, f = (i0 * K3[1] + i1) * K3[2] + i2;
                for (int c = 0; c < nc; c++) kbuf[o * nc + c] = k[f * nc + c];
            }
    int64_t sshape[3];
    CPLX *ds, *ks_;
    long nspec;
    if (!is_complex) {
        int64_t h[3];
        memcpy(h, F, sizeof(h));
        h[rank - 1] = F[rank - 1] / 2 + 1;
        nspec = prod(h, rank);
        ds = malloc(sizeof(CPLX) * nspec);
        ks_ = malloc(sizeof(CPLX) * nspec);
        FN(real_forward)(rank, F, dbuf, ds, sshape, nth);
        FN(real_forward)(rank, F, kbuf, ks_, sshape, nth);
    } else {
        nspec = nF;
        ds = malloc(sizeof(CPLX) * nspec);
        ks_ = malloc(sizeof(CPLX) * nspec);
        FN(complex_transform)(rank, F, (CPLX *)dbuf, ds, sshape, 0, nth);
        FN(complex_transform)(rank, F, (CPLX *)kbuf, ks_, sshape, 0, nth);
    }
    {
        FN(mul_ctx) mc = {ds, ks_};
        par_for(nspec, nth < 1 ? 1 : nth, 32768, FN(mul_worker), &mc);
    }
    int64_t oshape[3];
    REAL *outF = malloc(sizeof(REAL) * nF * nc);
    if (!is_complex) FN(real_backward)(rank, sshape, ds, F[rank - 1], outF, oshape, nth);
    else FN(complex_transform)(rank, sshape, ds, (CPLX *)outF, oshape, 1, nth);
    /* crop + stride: slice [k_eff-1, pds) step s (mod.rs:282-289) */
    {
        long Y3[3], S3[3];
        to3(ys, rank, 1, Y3);
        to3(str, rank, 1, S3);
        long f = 0;
        for (long i0 = 0; i0 < Y3[0]; i0++)
            for (long i1 = 0; i1 < Y3[1]; i1++) {
                long row = ((E3[0] - 1 + i0 * S3[0]) * F3[1] + (E3[1] - 1 + i1 * S3[1])) * F3[2];
                for (long i2 = 0; i2 < Y3[2]; i2++, f++) {
                    long o = row + E3[2] - 1 + i2 * S3[2];
                    for (int c = 0; c < nc; c++) y[f * nc + c] = outF[o * nc + c];
                }
            }
    }
    free(dbuf); free(kbuf); free(ds); free(ks_); free(outF);
    return ORC_OK;
}

#undef CPLX
#undef PLAN
#undef FN
