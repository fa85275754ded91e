// C ABI of libndconv (include/ndconv.h): argument checks in the reference's
// order, canonicalisation to three axes, dispatch to the CUDA kernels.
#include <stdio.h>
#include <string.h>

#include <string>

#include "common.cuh"
#include "direct.h"
#include "fft.h"
#include "geometry.h"

#include <atomic>
#include <mutex>
#include <map>
#include <set>
#include <utility>

namespace {
thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};
}

void ndconv_count_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

extern "C" uint64_t ndconv_kernel_launches(void) { return g_launches.load(); }

namespace {
thread_local int32_t g_tune[NDCONV_TUNE_COUNT] = {};
}
int ndconv_tune(int knob) { return (knob >= 0 && knob < NDCONV_TUNE_COUNT) ? g_tune[knob] : 0; }
extern "C" int ndconv_set_tuning(int32_t knob, int32_t value) {
    if (knob < 0 || knob >= NDCONV_TUNE_COUNT || value < 0)
        return ndconv_fail(NDCONV_ERR_INVALID, "unknown tuning knob or negative value");
    g_tune[knob] = value;
    return NDCONV_OK;
}
extern "C" int32_t ndconv_get_tuning(int32_t knob) { return ndconv_tune(knob); }

// The attribute is a per-(device, kernel) maximum: it is only ever raised, so
// a launch with less shared memory never lowers it below what another launch
// of the same kernel with more shared memory was granted.
cudaError_t ndconv_allow_smem(const void *kernel, int bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, int> granted;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    auto key = std::make_pair(dev, kernel);
    auto it = granted.find(key);
    if (it != granted.end() && it->second >= bytes) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) granted[key] = bytes;
    return e;
}

int ndconv_fail(int status, const char *msg) {
    g_last_error = msg ? msg : "";
    return status;
}

namespace ndconv {

// ConvMode::unfold (src/conv/mod.rs:28-66) on the dilated kernel extent.
static int unfold(const ndconv_problem *p, int64_t pad[3][2], int64_t str[3]) {
    for (int i = 0; i < p->rank; i++) {
        const int64_t ke = p->kernel_shape[i] * p->dilation[i] - p->dilation[i] + 1;
        switch (p->conv_mode) {
        case NDCONV_MODE_FULL: pad[i][0] = pad[i][1] = ke - 1; str[i] = 1; break;
        case NDCONV_MODE_SAME:
            if (ke % 2 == 0) {
                pad[i][0] = (ke - 1) / 2 + 1;
                pad[i][1] = (ke - 1) / 2;
            } else {
                pad[i][0] = pad[i][1] = (ke - 1) / 2;
            }
            str[i] = 1;
            break;
        case NDCONV_MODE_VALID: pad[i][0] = pad[i][1] = 0; str[i] = 1; break;
        case NDCONV_MODE_CUSTOM:
            pad[i][0] = pad[i][1] = p->mode_padding[i][0];
            str[i] = p->mode_strides[i];
            break;
        case NDCONV_MODE_EXPLICIT:
            pad[i][0] = p->mode_padding[i][0];
            pad[i][1] = p->mode_padding[i][1];
            str[i] = p->mode_strides[i];
            break;
        default: return ndconv_fail(NDCONV_ERR_INVALID, "unknown conv mode");
        }
        if (pad[i][0] < 0 || pad[i][1] < 0) return ndconv_fail(NDCONV_ERR_INVALID, "negative padding");
        if (str[i] < 1) return ndconv_fail(NDCONV_ERR_INVALID, "stride must be >= 1");
    }
    return NDCONV_OK;
}

// Per-axis border kinds and constants for a PaddingMode
// (src/padding/mod.rs:84-153: Zeros/Const become constants on every side).
static int borders(const ndconv_problem *p, int ax, int kind[2], double val[2][2]) {
    switch (p->padding_mode) {
    case NDCONV_PAD_ZEROS:
        kind[0] = kind[1] = BK_CONST;
        val[0][0] = val[0][1] = val[1][0] = val[1][1] = 0;
        return NDCONV_OK;
    case NDCONV_PAD_CONST:
        kind[0] = kind[1] = BK_CONST;
        val[0][0] = val[1][0] = p->const_value[0];
        val[0][1] = val[1][1] = p->const_value[1];
        return NDCONV_OK;
    case NDCONV_PAD_REFLECT: kind[0] = kind[1] = BK_REFLECT; break;
    case NDCONV_PAD_REPLICATE: kind[0] = kind[1] = BK_REPLICATE; break;
    case NDCONV_PAD_CIRCULAR: kind[0] = kind[1] = BK_CIRCULAR; break;
    case NDCONV_PAD_CUSTOM:
    case NDCONV_PAD_EXPLICIT:
        for (int s = 0; s < 2; s++) {
            const int src = (p->padding_mode == NDCONV_PAD_CUSTOM) ? 0 : s;
            const int b = p->border_kind[ax][src];
            switch (b) {
            case NDCONV_BORDER_ZEROS: kind[s] = BK_CONST; val[s][0] = val[s][1] = 0; break;
            case NDCONV_BORDER_CONST:
                kind[s] = BK_CONST;
                val[s][0] = p->border_value[ax][src][0];
                val[s][1] = p->border_value[ax][src][1];
                break;
            case NDCONV_BORDER_REFLECT: kind[s] = BK_REFLECT; break;
            case NDCONV_BORDER_REPLICATE: kind[s] = BK_REPLICATE; break;
            case NDCONV_BORDER_CIRCULAR: kind[s] = BK_CIRCULAR; break;
            default: return ndconv_fail(NDCONV_ERR_INVALID, "unknown border type");
            }
        }
        return NDCONV_OK;
    default: return ndconv_fail(NDCONV_ERR_INVALID, "unknown padding mode");
    }
    val[0][0] = val[0][1] = val[1][0] = val[1][1] = 0;
    return NDCONV_OK;
}

int plan_problem(const ndconv_problem *p, int algo, Plan3 *out) {
    if (!p) return ndconv_fail(NDCONV_ERR_INVALID, "null problem");
    if (p->rank < 1) return ndconv_fail(NDCONV_ERR_INVALID, "rank must be at least 1");
    // the crate is generic over any const N and any NumAssign element type
    // (src/conv/mod.rs:78-83,118-124); this library's kernels take ranks 1..3
    // and the element types of ndconv_dtype: everything else is refused,
    // never run on a fallback
    if (p->rank > 3) return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "rank above 3 is not supported (ranks 1..3)");
    if (p->dtype < NDCONV_F32 || p->dtype > NDCONV_U64)
        return ndconv_fail(NDCONV_ERR_UNSUPPORTED,
                           "element type not supported (f32, f64, c32, c64, i8, u8, i16, u16, i32, u32, i64, u64)");
    const int r = p->rank;
    for (int i = 0; i < r; i++) {
        if (p->data_shape[i] < 0 || p->kernel_shape[i] < 0)
            return ndconv_fail(NDCONV_ERR_INVALID, "negative extent");
        if (p->dilation[i] < 1) return ndconv_fail(NDCONV_ERR_INVALID, "dilation must be >= 1");
    }
    int64_t nx = 1, nk = 1;
    for (int i = 0; i < r; i++) {
        nx *= p->data_shape[i];
        nk *= p->kernel_shape[i];
    }
    // src/conv/mod.rs:136-144 / src/conv_fft/mod.rs:205-213
    if (nx == 0) return ndconv_fail(NDCONV_ERR_DATA_SHAPE, "Data shape shouldn't have ZERO");
    if (nk == 0) {
        if (algo == 1) return ndconv_fail(NDCONV_ERR_DATA_SHAPE, "Data shape shouldn't have ZERO (kernel)");
        return ndconv_fail(NDCONV_ERR_KERNEL_SHAPE, "Kernel shape shouldn't have ZERO");
    }
    int64_t pad[3][2], str[3];
    int s = unfold(p, pad, str);
    if (s) return s;
    Plan3 P{};
    P.rank = r;
    // canonical axes: rank-r problem in the last r slots
    const int off = 3 - r;
    for (int a = 0; a < 3; a++) {
        AxisGeom &A = P.ax[a];
        A = AxisGeom{};
        A.n = 1; A.p0 = 0; A.p1 = 0; A.L = 1; A.kf = A.kb = BK_CONST; A.K = 1; A.d = 1; A.keff = 1;
        A.s = 1; A.out = 1; A.xs = 0; A.ks = 0;
        P.cval[a][0][0] = P.cval[a][0][1] = P.cval[a][1][0] = P.cval[a][1][1] = 0;
    }
    bool data_contig = true, ker_contig = true;
    for (int i = 0; i < r; i++) {
        if (p->data_strides[i] != 0) data_contig = false;
        if (p->kernel_strides[i] != 0) ker_contig = false;
    }
    int64_t cs = 1, kcs = 1;
    for (int i = r - 1; i >= 0; i--) {
        AxisGeom &A = P.ax[off + i];
        A.n = p->data_shape[i];
        A.p0 = pad[i][0];
        A.p1 = pad[i][1];
        A.L = A.n + A.p0 + A.p1;
        A.K = p->kernel_shape[i];
        A.d = p->dilation[i];
        A.keff = A.K * A.d - A.d + 1;
        A.s = str[i];
        A.xs = data_contig ? cs : p->data_strides[i];
        A.ks = ker_contig ? kcs : p->kernel_strides[i];
        cs *= A.n;
        kcs *= A.K;
        int kind[2];
        double val[2][2];
        if ((s = borders(p, i, kind, val))) return s;
        A.kf = kind[0];
        A.kb = kind[1];
        for (int sd = 0; sd < 2; sd++)
            for (int c = 0; c < 2; c++) P.cval[off + i][sd][c] = val[sd][c];
    }
    // the reference panics where reflect indices leave the buffer
    // (src/padding/half_dim.rs:198-209 front, :245-256 back)
    int pad_err = 0;
    for (int a = off; a < 3; a++) {
        const AxisGeom &A = P.ax[a];
        if (A.kf == BK_REFLECT && A.p0 > 0 && 2 * A.p0 >= A.L) pad_err = 1;
        if (A.kb == BK_REFLECT && A.p1 > 0 && A.p1 >= A.p0 + A.n) pad_err = 1;
    }
    int mismatch = 0;
    for (int a = off; a < 3; a++)
        if (P.ax[a].keff > P.ax[a].L) mismatch = 1;
    // direct: padding (may panic) happens before the size check
    // (src/conv/mod.rs:149-158); FFT: size check first (src/conv_fft/mod.rs:218-227)
    if (algo == 0) {
        if (pad_err) return ndconv_fail(NDCONV_ERR_PAD_OUT_OF_RANGE, "reflect padding index out of range");
        if (mismatch) return ndconv_fail(NDCONV_ERR_MISMATCH_SHAPE, "ConvMode does not match KernelWithDilation size");
    } else {
        if (mismatch) return ndconv_fail(NDCONV_ERR_MISMATCH_SHAPE, "ConvMode does not match KernelWithDilation size");
        if (pad_err) return ndconv_fail(NDCONV_ERR_PAD_OUT_OF_RANGE, "reflect padding index out of range");
    }
    for (int a = 0; a < 3; a++) {
        AxisGeom &A = P.ax[a];
        A.out = (A.L - A.keff) / A.s + 1;  // src/conv/mod.rs:162-168
    }
    P.reverse = p->reverse ? 1 : 0;
    P.dtype = p->dtype;
    *out = P;
    return NDCONV_OK;
}

}  // namespace ndconv

using namespace ndconv;

extern "C" int ndconv_output_shape(const ndconv_problem *p, int32_t algo, int64_t out_shape[3]) {
    Plan3 P;
    int s = plan_problem(p, algo, &P);
    if (s) return s;
    if (out_shape)
        for (int i = 0; i < p->rank; i++) out_shape[i] = P.ax[3 - p->rank + i].out;
    return NDCONV_OK;
}

extern "C" int ndconv_padded_host(const ndconv_problem *p, const double *x, int32_t nc, double *out) {
    Plan3 P;
    int s = plan_problem(p, 0, &P);
    if (s) return s;
    if (!x || !out || (nc != 1 && nc != 2)) return ndconv_fail(NDCONV_ERR_INVALID, "null pointer or nc not 1 or 2");
    const AxisGeom *A = P.ax;
    int64_t u = 0;
    for (int64_t i0 = 0; i0 < A[0].L; i0++) {
        const int64_t m0 = axis_map(A[0], i0);
        for (int64_t i1 = 0; i1 < A[1].L; i1++) {
            const int64_t m1 = axis_map(A[1], i1);
            for (int64_t i2 = 0; i2 < A[2].L; i2++, u++) {
                const int64_t m2 = axis_map(A[2], i2);
                // the rule of resolve_padded: the last axis' constant first, then
                // the middle and leading axes', then pre-fill, else the sample
                const int64_t m[3] = {m0, m1, m2};
                const double *v = nullptr;
                double zero[2] = {0.0, 0.0};
                for (int a = 2; a >= 0 && !v; a--)
                    if (m[a] <= MAP_CONST_FRONT) v = P.cval[a][m[a] == MAP_CONST_FRONT ? 0 : 1];
                if (!v && (m0 < 0 || m1 < 0 || m2 < 0)) v = zero;
                if (!v) v = x + nc * (m0 * A[0].xs + m1 * A[1].xs + m2 * A[2].xs);
                for (int c = 0; c < nc; c++) out[nc * u + c] = v[c];
            }
        }
    }
    return NDCONV_OK;
}

extern "C" int ndconv_conv(const ndconv_problem *p, const void *data, const void *kernel, void *out,
                           void *stream) {
    Plan3 P;
    int s = plan_problem(p, 0, &P);
    if (s) return s;
    if (!data || !kernel || !out) return ndconv_fail(NDCONV_ERR_INVALID, "null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    switch (P.dtype) {
    case NDCONV_F32: e = direct_conv_launch<float>((const float *)data, (const float *)kernel, (float *)out, P.direct<float>(), st, 0); break;
    case NDCONV_F64: e = direct_conv_launch<double>((const double *)data, (const double *)kernel, (double *)out, P.direct<double>(), st, 0); break;
    case NDCONV_I32: e = direct_conv_launch<int32_t>((const int32_t *)data, (const int32_t *)kernel, (int32_t *)out, P.direct<int32_t>(), st, 0); break;
    case NDCONV_C32: e = direct_conv_launch<c32>((const c32 *)data, (const c32 *)kernel, (c32 *)out, P.direct<c32>(), st, 0); break;
    case NDCONV_C64: e = direct_conv_launch<c64>((const c64 *)data, (const c64 *)kernel, (c64 *)out, P.direct<c64>(), st, 0); break;
    // u32 and u64 share i32 and i64 bit for bit (wrapping sums)
    case NDCONV_U32: e = direct_conv_launch<int32_t>((const int32_t *)data, (const int32_t *)kernel, (int32_t *)out, P.direct<int32_t>(), st, 0); break;
    case NDCONV_I64:
    case NDCONV_U64: e = direct_conv_launch<int64_t>((const int64_t *)data, (const int64_t *)kernel, (int64_t *)out, P.direct<int64_t>(), st, 0); break;
    default: return conv_narrow_int(P, data, kernel, out, st);
    }
    if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
    return NDCONV_OK;
}

extern "C" int ndconv_conv_fft(const ndconv_problem *p, const void *data, const void *kernel, void *out,
                               ndconv_fft_processor *proc, void *stream) {
    Plan3 P;
    int s = plan_problem(p, 1, &P);
    if (s) return s;
    if (!data || !kernel || !out) return ndconv_fail(NDCONV_ERR_INVALID, "null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    int s2 = NDCONV_OK;
    switch (P.dtype) {
    case NDCONV_F32: s2 = conv_fft_run<float>(P.geom<float>(), P.reverse, (const float *)data, (const float *)kernel, (float *)out, proc, st, nullptr, 0); break;
    case NDCONV_F64: s2 = conv_fft_run<double>(P.geom<double>(), P.reverse, (const double *)data, (const double *)kernel, (double *)out, proc, st, nullptr, 0); break;
    case NDCONV_C32: s2 = conv_fft_run<c32>(P.geom<c32>(), P.reverse, (const c32 *)data, (const c32 *)kernel, (c32 *)out, proc, st, nullptr, 0); break;
    case NDCONV_C64: s2 = conv_fft_run<c64>(P.geom<c64>(), P.reverse, (const c64 *)data, (const c64 *)kernel, (c64 *)out, proc, st, nullptr, 0); break;
    default: return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "integer FFT convolution is not supported (documented broken upstream)");
    }
    if (s2 != NDCONV_ERR_UNSUPPORTED) return s2;
    // FFT lengths beyond one CTA's shared memory: the same convolution by the
    // direct kernel (results within the FFT path's tolerance)
    cudaError_t e = cudaSuccess;
    switch (P.dtype) {
    case NDCONV_F32: e = direct_conv_launch<float>((const float *)data, (const float *)kernel, (float *)out, P.direct<float>(), st, 0); break;
    case NDCONV_F64: e = direct_conv_launch<double>((const double *)data, (const double *)kernel, (double *)out, P.direct<double>(), st, 0); break;
    case NDCONV_C32: e = direct_conv_launch<c32>((const c32 *)data, (const c32 *)kernel, (c32 *)out, P.direct<c32>(), st, 0); break;
    default: e = direct_conv_launch<c64>((const c64 *)data, (const c64 *)kernel, (c64 *)out, P.direct<c64>(), st, 0); break;
    }
    if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
    return NDCONV_OK;
}

namespace {
int fft_variant_of(int32_t algo) {
    switch (algo) {
    case NDCONV_ALGO_FFT_ND: return FFTV_ND;
    case NDCONV_ALGO_FFT_RS: return FFTV_RS;
    case NDCONV_ALGO_FFT_ND_POW2: return FFTV_ND_POW2;
    case NDCONV_ALGO_FFT_RS_POW2: return FFTV_RS_POW2;
    default: return FFTV_AUTO;
    }
}
}  // namespace

extern "C" int ndconv_conv_algo(const ndconv_problem *p, int32_t algo, const void *data, const void *kernel,
                                void *out, void *stream) {
    if (algo == NDCONV_ALGO_DIRECT) return ndconv_conv(p, data, kernel, out, stream);
    if (algo == NDCONV_ALGO_FFT) return ndconv_conv_fft(p, data, kernel, out, nullptr, stream);
    if (algo == NDCONV_ALGO_DIRECT_BF16X3) return ndconv_conv_bf16x3(p, data, kernel, out, stream);
    if (algo < 0 || algo >= NDCONV_ALGO_COUNT) return ndconv_fail(NDCONV_ERR_INVALID, "unknown algorithm variant");
    Plan3 P;
    int s = plan_problem(p, 1, &P);
    if (s) return s;
    if (!data || !kernel || !out) return ndconv_fail(NDCONV_ERR_INVALID, "null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    const int fv = fft_variant_of(algo);
    switch (P.dtype) {
    case NDCONV_F32: return conv_fft_run<float>(P.geom<float>(), P.reverse, (const float *)data, (const float *)kernel, (float *)out, nullptr, st, nullptr, 0, fv);
    case NDCONV_F64: return conv_fft_run<double>(P.geom<double>(), P.reverse, (const double *)data, (const double *)kernel, (double *)out, nullptr, st, nullptr, 0, fv);
    case NDCONV_C32: return conv_fft_run<c32>(P.geom<c32>(), P.reverse, (const c32 *)data, (const c32 *)kernel, (c32 *)out, nullptr, st, nullptr, 0, fv);
    case NDCONV_C64: return conv_fft_run<c64>(P.geom<c64>(), P.reverse, (const c64 *)data, (const c64 *)kernel, (c64 *)out, nullptr, st, nullptr, 0, fv);
    default: return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "integer FFT convolution is not supported (documented broken upstream)");
    }
}

extern "C" int ndconv_fft_processor_bake(ndconv_fft_processor *proc, const ndconv_problem *p, const void *kernel,
                                         void *stream) {
    if (!proc || !kernel) return ndconv_fail(NDCONV_ERR_INVALID, "null argument");
    Plan3 P;
    int s = plan_problem(p, 1, &P);
    if (s) return s;
    if (P.dtype != ndconv_proc_dtype(proc)) return ndconv_fail(NDCONV_ERR_INVALID, "processor element type differs");
    cudaStream_t st = (cudaStream_t)stream;
    switch (P.dtype) {
    case NDCONV_F32: return conv_fft_bake<float>(P.geom<float>(), P.reverse, (const float *)kernel, proc, st);
    case NDCONV_F64: return conv_fft_bake<double>(P.geom<double>(), P.reverse, (const double *)kernel, proc, st);
    case NDCONV_C32: return conv_fft_bake<c32>(P.geom<c32>(), P.reverse, (const c32 *)kernel, proc, st);
    case NDCONV_C64: return conv_fft_bake<c64>(P.geom<c64>(), P.reverse, (const c64 *)kernel, proc, st);
    default: return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "integer FFT convolution is not supported");
    }
}

extern "C" int ndconv_conv_batch(const ndconv_problem *p, int64_t n, const void *const *data,
                                 const void *const *kernel, void *const *out, void *stream) {
    Plan3 P;
    int s = plan_problem(p, 0, &P);
    if (s) return s;
    if (n < 0) return ndconv_fail(NDCONV_ERR_INVALID, "negative batch size");
    if (n == 0) return NDCONV_OK;
    if (!data || !kernel || !out) return ndconv_fail(NDCONV_ERR_INVALID, "null pointer array");
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    switch (P.dtype) {
    case NDCONV_F32: e = direct_conv_batch_launch<float>(n, (const float *const *)data, (const float *const *)kernel, (float *const *)out, P.direct<float>(), st); break;
    case NDCONV_F64: e = direct_conv_batch_launch<double>(n, (const double *const *)data, (const double *const *)kernel, (double *const *)out, P.direct<double>(), st); break;
    case NDCONV_I32: e = direct_conv_batch_launch<int32_t>(n, (const int32_t *const *)data, (const int32_t *const *)kernel, (int32_t *const *)out, P.direct<int32_t>(), st); break;
    case NDCONV_C32: e = direct_conv_batch_launch<c32>(n, (const c32 *const *)data, (const c32 *const *)kernel, (c32 *const *)out, P.direct<c32>(), st); break;
    case NDCONV_C64: e = direct_conv_batch_launch<c64>(n, (const c64 *const *)data, (const c64 *const *)kernel, (c64 *const *)out, P.direct<c64>(), st); break;
    default: return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "this integer element type runs ndconv_conv only");
    }
    if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
    return NDCONV_OK;
}

extern "C" int ndconv_conv_fft_batch(const ndconv_problem *p, int64_t n, const void *const *data,
                                     const void *const *kernel, void *const *out, ndconv_fft_processor *proc,
                                     void *stream) {
    Plan3 P;
    int s = plan_problem(p, 1, &P);
    if (s) return s;
    if (n < 0) return ndconv_fail(NDCONV_ERR_INVALID, "negative batch size");
    if (n == 0) return NDCONV_OK;
    if (!data || !kernel || !out) return ndconv_fail(NDCONV_ERR_INVALID, "null pointer array");
    cudaStream_t st = (cudaStream_t)stream;
    switch (P.dtype) {
    case NDCONV_F32: return conv_fft_batch_run<float>(P.geom<float>(), P.reverse, n, (const float *const *)data, (const float *const *)kernel, (float *const *)out, proc, st);
    case NDCONV_F64: return conv_fft_batch_run<double>(P.geom<double>(), P.reverse, n, (const double *const *)data, (const double *const *)kernel, (double *const *)out, proc, st);
    case NDCONV_C32: return conv_fft_batch_run<c32>(P.geom<c32>(), P.reverse, n, (const c32 *const *)data, (const c32 *const *)kernel, (c32 *const *)out, proc, st);
    case NDCONV_C64: return conv_fft_batch_run<c64>(P.geom<c64>(), P.reverse, n, (const c64 *const *)data, (const c64 *const *)kernel, (c64 *const *)out, proc, st);
    default: return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "integer FFT convolution is not supported (documented broken upstream)");
    }
}

static int check_proc_shape(ndconv_fft_processor *proc, int32_t rank, const int64_t shape[3]) {
    if (!proc) return ndconv_fail(NDCONV_ERR_INVALID, "null processor");
    if (rank < 1 || rank > 3) return ndconv_fail(NDCONV_ERR_INVALID, "rank must be 1..3");
    for (int i = 0; i < rank; i++)
        if (shape[i] < 1) return ndconv_fail(NDCONV_ERR_INVALID, "empty axis");
    return NDCONV_OK;
}

extern "C" int ndconv_fft_forward(ndconv_fft_processor *proc, int32_t rank, const int64_t shape[3],
                                  const void *in, void *out, int64_t out_shape[3], void *stream) {
    int s = check_proc_shape(proc, rank, shape);
    if (s) return s;
    const int dt = ndconv_proc_dtype(proc);
    const bool real = (dt == NDCONV_F32 || dt == NDCONV_F64);
    // rotated layout (src/conv_fft/processor/real.rs:133-153): 1-D (h), 2-D (h, d0), 3-D (d1, h, d0)
    int64_t osh[3] = {0, 0, 0};
    const int64_t h = real ? shape[rank - 1] / 2 + 1 : shape[rank - 1];
    if (rank == 1) {
        osh[0] = h;
    } else if (rank == 2) {
        osh[0] = h;
        osh[1] = shape[0];
    } else {
        osh[0] = shape[1];
        osh[1] = h;
        osh[2] = shape[0];
    }
    if (out_shape)
        for (int i = 0; i < rank; i++) out_shape[i] = osh[i];
    if (!out) return NDCONV_OK;
    if (!in) return ndconv_fail(NDCONV_ERR_INVALID, "null input");
    cudaStream_t st = (cudaStream_t)stream;
    switch (dt) {
    case NDCONV_F32: return proc_forward<float>(proc, rank, shape, (const float *)in, (c32 *)out, st);
    case NDCONV_F64: return proc_forward<double>(proc, rank, shape, (const double *)in, (c64 *)out, st);
    case NDCONV_C32: return proc_forward<c32>(proc, rank, shape, (const c32 *)in, (c32 *)out, st);
    default: return proc_forward<c64>(proc, rank, shape, (const c64 *)in, (c64 *)out, st);
    }
}

extern "C" int ndconv_fft_backward(ndconv_fft_processor *proc, int32_t rank, const int64_t shape[3],
                                   const void *in, void *out, int64_t out_shape[3], void *stream) {
    int s = check_proc_shape(proc, rank, shape);
    if (s) return s;
    const int dt = ndconv_proc_dtype(proc);
    int64_t osh[3] = {0, 0, 0};
    if (!out) {
        // shape query only
        int64_t nat[3];
        if (rank == 1) nat[0] = shape[0];
        else {
            nat[0] = shape[rank - 1];
            for (int i = 1; i < rank; i++) nat[i] = shape[i - 1];
        }
        if (dt == NDCONV_F32 || dt == NDCONV_F64) nat[rank - 1] = ndconv_proc_origin_len(proc);
        if (out_shape)
            for (int i = 0; i < rank; i++) out_shape[i] = nat[i];
        return NDCONV_OK;
    }
    if (!in) return ndconv_fail(NDCONV_ERR_INVALID, "null input");
    cudaStream_t st = (cudaStream_t)stream;
    switch (dt) {
    case NDCONV_F32: s = proc_backward<float>(proc, rank, shape, (const c32 *)in, (float *)out, osh, st); break;
    case NDCONV_F64: s = proc_backward<double>(proc, rank, shape, (const c64 *)in, (double *)out, osh, st); break;
    case NDCONV_C32: s = proc_backward<c32>(proc, rank, shape, (const c32 *)in, (c32 *)out, osh, st); break;
    default: s = proc_backward<c64>(proc, rank, shape, (const c64 *)in, (c64 *)out, osh, st); break;
    }
    if (out_shape)
        for (int i = 0; i < rank; i++) out_shape[i] = osh[i];
    return s;
}

extern "C" const char *ndconv_last_error(void) { return g_last_error.c_str(); }

extern "C" const char *ndconv_version(void) { return "ndconv-gb300 0.1.0 (sm_103a)"; }
