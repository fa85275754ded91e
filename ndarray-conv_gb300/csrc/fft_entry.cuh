// conv_fft entry points (run, bake, batched waves, scratch size) and the
// FFT processor's forward / backward, as templates over the element type;
// fft_<type>.cu instantiate them (NDCONV_INST_FFT / NDCONV_INST_PROC).
#pragma once
#include "fft_kernels.cuh"

namespace ndconv {

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

#define NDCONV_INST_FFT(T)                                                                          \
    template int conv_fft_run<T>(const Geom3<T> &, int, const T *, const T *, T *,                \
                                 ndconv_fft_processor *, cudaStream_t, void *, size_t, int);     \
    template int conv_fft_batch_run<T>(const Geom3<T> &, int, int64_t, const T *const *,          \
                                       const T *const *, T *const *, ndconv_fft_processor *,      \
                                       cudaStream_t, int);                                         \
    template size_t conv_fft_scratch_bytes<T>(const Geom3<T> &, int);                              \
    template int conv_fft_bake<T>(const Geom3<T> &, int, const T *, ndconv_fft_processor *, cudaStream_t);

#define NDCONV_INST_PROC(T)                                                                          \
    template int proc_forward<T>(ndconv_fft_processor *, int, const int64_t *, const T *,          \
                                 CplxT<Elem<T>::Real>::type *, cudaStream_t);                       \
    template int proc_backward<T>(ndconv_fft_processor *, int, const int64_t *,                     \
                                  const CplxT<Elem<T>::Real>::type *, T *, int64_t *, cudaStream_t);

}  // namespace ndconv
