// Direct N-d convolution (ConvExt::conv, src/conv/mod.rs:128-200) on sm_103a.
//
// One CTA computes a TY x TX tile of one output plane.  The padded input
// is never materialised: for every chunk of kernel taps the CTA stages the
// window of the padded input it needs in shared memory, evaluating each
// padded position with the closed-form border map (axis_map) straight from
// the unpadded data, then every thread accumulates RX outputs of one row
// (columns tx, tx+BX, ...) over the chunk's taps.  Taps follow the
// reference's order (row-major over the reversed kernel, dilation as the
// tap stride), and exact-zero taps are skipped like gen_offset_list
// (src/dilation/mod.rs:47-50); the skip is warp-uniform.
#include "common.cuh"
#include "direct.h"

namespace ndconv {

template <typename T, int RX>
__global__ void __launch_bounds__(256) direct_tile_kernel(const T *__restrict__ x,
                                                          const T *__restrict__ k,
                                                          T *__restrict__ y, DirectParams<T> P) {
    using E = Elem<T>;
    using Acc = typename E::Acc;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geom3<T> &g = P.g;
    const AxisGeom &A0 = g.ax[0], &A1 = g.ax[1], &A2 = g.ax[2];
    const int BX = blockDim.x, BY = blockDim.y;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * BX + tx, nthr = BX * BY;
    const int TX = BX * RX;

    T *tile = reinterpret_cast<T *>(smem_raw);
    T *wsm = tile + P.tile_elems;
    int64_t *mrow = reinterpret_cast<int64_t *>(smem_raw + P.maps_off);
    int64_t *mcol = mrow + P.max_rows;

    const int64_t oz = blockIdx.z;
    const int64_t oy0 = (int64_t)blockIdx.y * BY;
    const int64_t ox0 = (int64_t)blockIdx.x * TX;

    Acc acc[RX];
#pragma unroll
    for (int r = 0; r < RX; r++) acc[r] = E::zero();

    const int64_t s1 = A1.s, s2 = A2.s, d1 = A1.d, d2 = A2.d;
    for (int64_t kz = 0; kz < A0.K; kz++) {
        const int64_t mz = axis_map(A0, oz * A0.s + kz * A0.d);
        const int64_t kzs = tap_source(kz, A0.K, P.reverse);
        for (int64_t ky0 = 0; ky0 < A1.K; ky0 += P.cky) {
            const int cky = (int)(P.cky < A1.K - ky0 ? P.cky : A1.K - ky0);
            const int64_t row0 = oy0 * s1 + ky0 * d1;
            const int nrows = (int)((BY - 1) * s1 + (cky - 1) * d1 + 1);
            for (int64_t kx0 = 0; kx0 < A2.K; kx0 += P.ckx) {
                const int ckx = (int)(P.ckx < A2.K - kx0 ? P.ckx : A2.K - kx0);
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
        T *yrow = y + (oz * A1.out + oy) * A2.out;
#pragma unroll
        for (int r = 0; r < RX; r++) {
            const int64_t ox = ox0 + tx + (int64_t)r * BX;
            if (ox < A2.out) yrow[ox] = E::out(acc[r]);
        }
    }
}

// One thread per output, reading the data through the border map with no
// staging.  Used when a tile would not fit in shared memory (very large
// strides); correct for every geometry.
template <typename T>
__global__ void __launch_bounds__(256) direct_naive_kernel(const T *__restrict__ x,
                                                           const T *__restrict__ k,
                                                           T *__restrict__ y, DirectParams<T> P) {
    using E = Elem<T>;
    using Acc = typename E::Acc;
    const Geom3<T> &g = P.g;
    const AxisGeom &A0 = g.ax[0], &A1 = g.ax[1], &A2 = g.ax[2];
    const int64_t total = A0.out * A1.out * A2.out;
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < total;
         o += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ox = o % A2.out, oy = (o / A2.out) % A1.out, oz = o / (A2.out * A1.out);
        Acc acc = E::zero();
        for (int64_t kz = 0; kz < A0.K; kz++) {
            const int64_t mz = axis_map(A0, oz * A0.s + kz * A0.d);
            const int64_t kzs = tap_source(kz, A0.K, P.reverse);
            for (int64_t ky = 0; ky < A1.K; ky++) {
                const int64_t my = axis_map(A1, oy * A1.s + ky * A1.d);
                const int64_t kys = tap_source(ky, A1.K, P.reverse);
                for (int64_t kx = 0; kx < A2.K; kx++) {
                    const T w = k[kzs * A0.ks + kys * A1.ks + tap_source(kx, A2.K, P.reverse) * A2.ks];
                    if (E::is_zero(w)) continue;
                    const int64_t mx = axis_map(A2, ox * A2.s + kx * A2.d);
                    E::mac(acc, resolve_padded<T>(x, g, mz, my, mx), w);
                }
            }
        }
        y[o] = E::out(acc);
    }
}

namespace {
constexpr int kMaxCols = 2048;
constexpr size_t kSmemBudget = 96 * 1024;

template <typename T> size_t smem_bytes(const DirectParams<T> &P) {
    return (size_t)P.maps_off + sizeof(int64_t) * (P.max_rows + P.max_cols);
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
        int64_t ckx = A2.K;
        if (base_cols + (ckx - 1) * A2.d > kMaxCols) ckx = (kMaxCols - base_cols) / A2.d + 1;
        if (ckx < 1) continue;
        const int64_t W = base_cols + (ckx - 1) * A2.d;
        const int64_t base_rows = (int64_t)(BY - 1) * A1.s + 1;
        // largest cky whose window fits the budget
        int64_t cky = A1.K;
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
        return true;
    }
    return false;
}

template <typename T, int RX> cudaError_t launch_tile(const T *x, const T *k, T *y, const DirectParams<T> &P,
                                                      int BX, int BY, cudaStream_t st) {
    const size_t sm = smem_bytes(P);
    auto fn = direct_tile_kernel<T, RX>;
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kSmemBudget + 4096);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const AxisGeom &A0 = P.g.ax[0], &A1 = P.g.ax[1], &A2 = P.g.ax[2];
    const int64_t TX = (int64_t)BX * RX;
    dim3 grid((unsigned)((A2.out + TX - 1) / TX), (unsigned)((A1.out + BY - 1) / BY), (unsigned)A0.out);
    fn<<<grid, dim3(BX, BY), sm, st>>>(x, k, y, P);
    ndconv_count_launch();
    return cudaGetLastError();
}
}  // namespace

template <typename T>
cudaError_t direct_conv_launch(const T *x, const T *k, T *y, DirectParams<T> P, cudaStream_t st,
                               int force_naive) {
    const AxisGeom &A0 = P.g.ax[0], &A1 = P.g.ax[1], &A2 = P.g.ax[2];
    if (A0.out <= 0 || A1.out <= 0 || A2.out <= 0) return cudaSuccess;
    int BX = 0, BY = 0;
    const bool grid_ok = A0.out < 65536 && (A1.out + 7) / 8 < 65536;
    if (!force_naive && grid_ok) {
        const int RX = 4;
        if (plan_tile(P, RX, BX, BY)) return launch_tile<T, 4>(x, k, y, P, BX, BY, st);
        if (plan_tile(P, 1, BX, BY)) return launch_tile<T, 1>(x, k, y, P, BX, BY, st);
    }
    const int64_t total = A0.out * A1.out * A2.out;
    int64_t blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    direct_naive_kernel<T><<<(unsigned)blocks, 256, 0, st>>>(x, k, y, P);
    ndconv_count_launch();
    return cudaGetLastError();
}

template cudaError_t direct_conv_launch<float>(const float *, const float *, float *, DirectParams<float>,
                                               cudaStream_t, int);
template cudaError_t direct_conv_launch<double>(const double *, const double *, double *,
                                                DirectParams<double>, cudaStream_t, int);
template cudaError_t direct_conv_launch<int32_t>(const int32_t *, const int32_t *, int32_t *,
                                                 DirectParams<int32_t>, cudaStream_t, int);
template cudaError_t direct_conv_launch<c32>(const c32 *, const c32 *, c32 *, DirectParams<c32>,
                                             cudaStream_t, int);
template cudaError_t direct_conv_launch<c64>(const c64 *, const c64 *, c64 *, DirectParams<c64>,
                                             cudaStream_t, int);

}  // namespace ndconv
