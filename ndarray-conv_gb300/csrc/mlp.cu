// Learned dispatcher network: a small MLP (n_in -> H -> H -> n_out, ReLU)
// that maps shape/mode features of a convolution to predicted log-time per
// algorithm variant.  Forward, backward (masked mean-squared error) and Adam
// run as hand-written CUDA kernels; no counterpart in the reference crate.
//
// Parameters live in one flat f32 device array:
//   W1[H][n_in], b1[H], W2[H][H], b2[H], W3[n_out][H], b3[n_out]
// Samples are processed in tiles of kTile rows per CTA with the layer
// activations of the tile in shared memory; weight gradients are summed
// per CTA and then reduced across CTAs in a fixed order (deterministic).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "common.cuh"
#include "ndconv.h"

namespace ndconv {
namespace mlp {

constexpr int kTile = 32;      // samples per CTA
constexpr int kThreads = 256;
constexpr int kMaxIn = 32, kMaxH = 64, kMaxOut = 16;

struct Dims {
    int in, h, out;
    __host__ __device__ int64_t w1() const { return 0; }
    __host__ __device__ int64_t b1() const { return (int64_t)h * in; }
    __host__ __device__ int64_t w2() const { return b1() + h; }
    __host__ __device__ int64_t b2() const { return w2() + (int64_t)h * h; }
    __host__ __device__ int64_t w3() const { return b2() + h; }
    __host__ __device__ int64_t b3() const { return w3() + (int64_t)out * h; }
    __host__ __device__ int64_t count() const { return b3() + out; }
};

// dst[r][j] = act(sum_i src[r][i] * W[j][i] + b[j]) for the tile's rows
__device__ __forceinline__ void dense(const float *__restrict__ W, const float *__restrict__ b,
                                      const float *src, int n_src, float *dst, int n_dst, int rows, bool relu) {
    for (int u = threadIdx.x; u < rows * n_dst; u += blockDim.x) {
        const int r = u / n_dst, j = u - r * n_dst;
        const float *s = src + r * n_src;
        const float *w = W + (int64_t)j * n_src;
        float acc = b[j];
        for (int i = 0; i < n_src; i++) acc = fmaf(s[i], w[i], acc);
        dst[u] = relu ? fmaxf(acc, 0.f) : acc;
    }
}

__global__ void __launch_bounds__(kThreads) forward_kernel(Dims d, const float *__restrict__ P,
                                                           const float *__restrict__ x, int64_t n,
                                                           float *__restrict__ y) {
    __shared__ float a0[kTile * kMaxIn], a1[kTile * kMaxH], a2[kTile * kMaxH];
    const int64_t r0 = (int64_t)blockIdx.x * kTile;
    const int rows = (int)(n - r0 < kTile ? n - r0 : kTile);
    for (int u = threadIdx.x; u < rows * d.in; u += blockDim.x) a0[u] = x[r0 * d.in + u];
    __syncthreads();
    dense(P + d.w1(), P + d.b1(), a0, d.in, a1, d.h, rows, true);
    __syncthreads();
    dense(P + d.w2(), P + d.b2(), a1, d.h, a2, d.h, rows, true);
    __syncthreads();
    for (int u = threadIdx.x; u < rows * d.out; u += blockDim.x) {
        const int r = u / d.out, o = u - r * d.out;
        const float *s = a2 + r * d.h;
        const float *w = P + d.w3() + (int64_t)o * d.h;
        float acc = P[d.b3() + o];
        for (int i = 0; i < d.h; i++) acc = fmaf(s[i], w[i], acc);
        y[(r0 + r) * d.out + o] = acc;
    }
}

// Per-CTA gradient of L = sum_{n,o} m (y - t)^2 / (2 * msum) over the
// tile's rows into part[blockIdx.x][count]; loss_part[blockIdx.x].
__global__ void __launch_bounds__(kThreads) backward_kernel(Dims d, const float *__restrict__ P,
                                                            const float *__restrict__ x,
                                                            const float *__restrict__ t,
                                                            const float *__restrict__ m, int64_t n,
                                                            const float *__restrict__ msum,
                                                            float *__restrict__ part,
                                                            float *__restrict__ loss_part) {
    __shared__ float a0[kTile * kMaxIn], a1[kTile * kMaxH], a2[kTile * kMaxH];
    __shared__ float g2[kTile * kMaxH], g3[kTile * kMaxOut];
    __shared__ float red[kThreads];
    const int64_t r0 = (int64_t)blockIdx.x * kTile;
    const int rows = (int)(n - r0 < kTile ? n - r0 : kTile);
    const float inv = 1.f / fmaxf(*msum, 1.f);
    for (int u = threadIdx.x; u < rows * d.in; u += blockDim.x) a0[u] = x[r0 * d.in + u];
    __syncthreads();
    dense(P + d.w1(), P + d.b1(), a0, d.in, a1, d.h, rows, true);
    __syncthreads();
    dense(P + d.w2(), P + d.b2(), a1, d.h, a2, d.h, rows, true);
    __syncthreads();
    // output layer and dL/dy
    float lsum = 0.f;
    for (int u = threadIdx.x; u < rows * d.out; u += blockDim.x) {
        const int r = u / d.out, o = u - r * d.out;
        const float *s = a2 + r * d.h;
        const float *w = P + d.w3() + (int64_t)o * d.h;
        float acc = P[d.b3() + o];
        for (int i = 0; i < d.h; i++) acc = fmaf(s[i], w[i], acc);
        const int64_t gi = (r0 + r) * d.out + o;
        const float mk = m[gi];
        const float e = (mk != 0.f) ? (acc - t[gi]) : 0.f;
        lsum += mk * e * e;
        g3[u] = mk * e * inv;
    }
    red[threadIdx.x] = lsum;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss_part[blockIdx.x] = 0.5f * red[0] * inv;
    float *G = part + (int64_t)blockIdx.x * d.count();
    // layer 3 weights
    for (int u = threadIdx.x; u < d.out * (d.h + 1); u += blockDim.x) {
        const int o = u / (d.h + 1), j = u - o * (d.h + 1);
        float acc = 0.f;
        if (j < d.h) {
            for (int r = 0; r < rows; r++) acc = fmaf(g3[r * d.out + o], a2[r * d.h + j], acc);
            G[d.w3() + (int64_t)o * d.h + j] = acc;
        } else {
            for (int r = 0; r < rows; r++) acc += g3[r * d.out + o];
            G[d.b3() + o] = acc;
        }
    }
    // back through layer 3 and ReLU 2
    for (int u = threadIdx.x; u < rows * d.h; u += blockDim.x) {
        const int r = u / d.h, j = u - r * d.h;
        float acc = 0.f;
        for (int o = 0; o < d.out; o++) acc = fmaf(g3[r * d.out + o], P[d.w3() + (int64_t)o * d.h + j], acc);
        g2[u] = a2[u] > 0.f ? acc : 0.f;
    }
    __syncthreads();
    for (int u = threadIdx.x; u < d.h * (d.h + 1); u += blockDim.x) {
        const int j = u / (d.h + 1), i = u - j * (d.h + 1);
        float acc = 0.f;
        if (i < d.h) {
            for (int r = 0; r < rows; r++) acc = fmaf(g2[r * d.h + j], a1[r * d.h + i], acc);
            G[d.w2() + (int64_t)j * d.h + i] = acc;
        } else {
            for (int r = 0; r < rows; r++) acc += g2[r * d.h + j];
            G[d.b2() + j] = acc;
        }
    }
    // back through layer 2 and ReLU 1 (g1 reuses a2's storage)
    float *g1 = a2;
    __syncthreads();
    for (int u = threadIdx.x; u < rows * d.h; u += blockDim.x) {
        const int r = u / d.h, i = u - r * d.h;
        float acc = 0.f;
        for (int j = 0; j < d.h; j++) acc = fmaf(g2[r * d.h + j], P[d.w2() + (int64_t)j * d.h + i], acc);
        g1[u] = a1[u] > 0.f ? acc : 0.f;
    }
    __syncthreads();
    for (int u = threadIdx.x; u < d.h * (d.in + 1); u += blockDim.x) {
        const int i = u / (d.in + 1), f = u - i * (d.in + 1);
        float acc = 0.f;
        if (f < d.in) {
            for (int r = 0; r < rows; r++) acc = fmaf(g1[r * d.h + i], a0[r * d.in + f], acc);
            G[d.w1() + (int64_t)i * d.in + f] = acc;
        } else {
            for (int r = 0; r < rows; r++) acc += g1[r * d.h + i];
            G[d.b1() + i] = acc;
        }
    }
}

// grad[p] = sum over CTAs of part[c][p] (fixed order); loss = sum of loss_part
__global__ void reduce_kernel(const float *__restrict__ part, const float *__restrict__ loss_part, int nblk,
                              int64_t count, float *__restrict__ grad, float *__restrict__ loss) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < count) {
        float acc = 0.f;
        for (int c = 0; c < nblk; c++) acc += part[(int64_t)c * count + p];
        grad[p] = acc;
    }
    if (p == 0 && loss) {
        float l = 0.f;
        for (int c = 0; c < nblk; c++) l += loss_part[c];
        *loss = l;
    }
}

// sum of the mask (the loss normaliser), one CTA
__global__ void mask_sum_kernel(const float *__restrict__ m, int64_t n, float *__restrict__ out) {
    __shared__ float red[kThreads];
    float acc = 0.f;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += m[i];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

// Adam (Kingma & Ba 2015) with bias correction folded into the step size
__global__ void adam_kernel(float *__restrict__ P, const float *__restrict__ g, float *__restrict__ m1,
                            float *__restrict__ m2, int64_t count, float lr_t, float b1, float b2, float eps) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= count) return;
    const float gi = g[p];
    const float a = b1 * m1[p] + (1.f - b1) * gi;
    const float v = b2 * m2[p] + (1.f - b2) * gi * gi;
    m1[p] = a;
    m2[p] = v;
    P[p] -= lr_t * a / (sqrtf(v) + eps);
}

// rows idx[i] of src (width w) -> dst row i
__global__ void gather_rows_kernel(const float *__restrict__ src, const int32_t *__restrict__ idx, int64_t n,
                                   int w, float *__restrict__ dst) {
    const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= n * w) return;
    const int64_t i = u / w;
    dst[u] = src[(int64_t)idx[i] * w + (u - i * w)];
}

}  // namespace mlp
}  // namespace ndconv

struct ndconv_mlp {
    ndconv::mlp::Dims d;
    int device = 0;
    float *P = nullptr;   // parameters
    float *m1 = nullptr;  // Adam moments
    float *m2 = nullptr;
    float *grad = nullptr;
    int64_t step = 0;
};

using namespace ndconv;
using namespace ndconv::mlp;

namespace {
int grad_into(ndconv_mlp *net, const float *x, const float *t, const float *m, int64_t n, float *grad,
              float *loss, cudaStream_t st) {
    const int nblk = (int)((n + kTile - 1) / kTile);
    const int64_t cnt = net->d.count();
    float *part = nullptr, *lp = nullptr, *msum = nullptr;
    NDCONV_CUDA_OK(cudaMallocAsync((void **)&part, sizeof(float) * (size_t)(nblk * cnt + nblk + 1), st));
    lp = part + (size_t)nblk * cnt;
    msum = lp + nblk;
    mask_sum_kernel<<<1, kThreads, 0, st>>>(m, n * net->d.out, msum);
    ndconv_count_launch();
    backward_kernel<<<nblk, kThreads, 0, st>>>(net->d, net->P, x, t, m, n, msum, part, lp);
    ndconv_count_launch();
    reduce_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, st>>>(part, lp, nblk, cnt, grad, loss);
    ndconv_count_launch();
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(part, st);
    if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
    return NDCONV_OK;
}
}  // namespace

extern "C" int ndconv_mlp_create(int32_t n_in, int32_t n_hidden, int32_t n_out, uint64_t seed, ndconv_mlp **out) {
    if (!out) return ndconv_fail(NDCONV_ERR_INVALID, "null output");
    if (n_in < 1 || n_in > kMaxIn || n_hidden < 1 || n_hidden > kMaxH || n_out < 1 || n_out > kMaxOut)
        return ndconv_fail(NDCONV_ERR_INVALID, "MLP sizes out of range (in <= 32, hidden <= 64, out <= 16)");
    auto *net = new ndconv_mlp();
    net->d = Dims{n_in, n_hidden, n_out};
    cudaGetDevice(&net->device);
    const int64_t cnt = net->d.count();
    // He-uniform initial weights, zero biases (host RNG, then one copy)
    std::vector<float> h((size_t)cnt, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int64_t off, int fan_out, int fan_in) {
        const float lim = std::sqrt(6.0f / (float)fan_in);
        std::uniform_real_distribution<float> u(-lim, lim);
        for (int64_t i = 0; i < (int64_t)fan_out * fan_in; i++) h[(size_t)(off + i)] = u(rng);
    };
    fill(net->d.w1(), n_hidden, n_in);
    fill(net->d.w2(), n_hidden, n_hidden);
    fill(net->d.w3(), n_out, n_hidden);
    cudaError_t e = cudaMalloc((void **)&net->P, sizeof(float) * 4 * (size_t)cnt);
    if (e != cudaSuccess) {
        delete net;
        return ndconv_fail(NDCONV_ERR_NO_MEMORY, cudaGetErrorString(e));
    }
    net->m1 = net->P + cnt;
    net->m2 = net->m1 + cnt;
    net->grad = net->m2 + cnt;
    cudaMemset(net->m1, 0, sizeof(float) * 3 * (size_t)cnt);
    cudaMemcpy(net->P, h.data(), sizeof(float) * (size_t)cnt, cudaMemcpyHostToDevice);
    *out = net;
    return NDCONV_OK;
}

extern "C" int ndconv_mlp_destroy(ndconv_mlp *net) {
    if (!net) return NDCONV_OK;
    cudaFree(net->P);
    delete net;
    return NDCONV_OK;
}

extern "C" int64_t ndconv_mlp_param_count(const ndconv_mlp *net) { return net ? net->d.count() : -1; }

extern "C" int ndconv_mlp_params(ndconv_mlp *net, float *host, int64_t n, int32_t set) {
    if (!net || !host) return ndconv_fail(NDCONV_ERR_INVALID, "null argument");
    if (n != net->d.count()) return ndconv_fail(NDCONV_ERR_INVALID, "parameter count mismatch");
    cudaError_t e = set ? cudaMemcpy(net->P, host, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice)
                        : cudaMemcpy(host, net->P, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
    if (set) {
        cudaMemset(net->m1, 0, sizeof(float) * 2 * (size_t)n);
        net->step = 0;
    }
    return NDCONV_OK;
}

extern "C" int ndconv_mlp_forward(ndconv_mlp *net, const float *x, int64_t n, float *y, void *stream) {
    if (!net || !x || !y) return ndconv_fail(NDCONV_ERR_INVALID, "null argument");
    if (n <= 0) return NDCONV_OK;
    cudaStream_t st = (cudaStream_t)stream;
    forward_kernel<<<(unsigned)((n + kTile - 1) / kTile), kThreads, 0, st>>>(net->d, net->P, x, n, y);
    ndconv_count_launch();
    NDCONV_CUDA_OK(cudaGetLastError());
    return NDCONV_OK;
}

extern "C" int ndconv_mlp_gradient(ndconv_mlp *net, const float *x, const float *t, const float *mask, int64_t n,
                                   float *grad, float *loss, void *stream) {
    if (!net || !x || !t || !mask || !grad) return ndconv_fail(NDCONV_ERR_INVALID, "null argument");
    if (n <= 0) return ndconv_fail(NDCONV_ERR_INVALID, "no samples");
    return grad_into(net, x, t, mask, n, grad, loss, (cudaStream_t)stream);
}

extern "C" int ndconv_mlp_train(ndconv_mlp *net, const float *x, const float *t, const float *mask, int64_t n,
                                int32_t epochs, int32_t batch, float lr, uint64_t seed, float *final_loss,
                                void *stream) {
    if (!net || !x || !t || !mask) return ndconv_fail(NDCONV_ERR_INVALID, "null argument");
    if (n <= 0 || epochs < 0 || batch < 1) return ndconv_fail(NDCONV_ERR_INVALID, "bad training arguments");
    cudaStream_t st = (cudaStream_t)stream;
    const Dims d = net->d;
    const int64_t cnt = d.count();
    const int64_t B = std::min<int64_t>(batch, n);
    // device minibatch buffers and a shuffled index list per epoch
    float *bx = nullptr;
    NDCONV_CUDA_OK(cudaMalloc((void **)&bx, sizeof(float) * (size_t)B * (d.in + 2 * d.out) + sizeof(float)));
    float *bt = bx + B * d.in, *bm = bt + B * d.out, *dloss = bm + B * d.out;
    int32_t *didx = nullptr;
    cudaError_t e = cudaMalloc((void **)&didx, sizeof(int32_t) * (size_t)n);
    if (e != cudaSuccess) {
        cudaFree(bx);
        return ndconv_fail(NDCONV_ERR_NO_MEMORY, cudaGetErrorString(e));
    }
    std::vector<int32_t> idx((size_t)n);
    for (int64_t i = 0; i < n; i++) idx[(size_t)i] = (int32_t)i;
    std::mt19937_64 rng(seed);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    int s = NDCONV_OK;
    for (int ep = 0; ep < epochs && s == NDCONV_OK; ep++) {
        std::shuffle(idx.begin(), idx.end(), rng);
        cudaMemcpyAsync(didx, idx.data(), sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, st);
        for (int64_t b0 = 0; b0 + B <= n; b0 += B) {
            const unsigned g1 = (unsigned)((B * d.in + 255) / 256), g2 = (unsigned)((B * d.out + 255) / 256);
            gather_rows_kernel<<<g1, 256, 0, st>>>(x, didx + b0, B, d.in, bx);
            gather_rows_kernel<<<g2, 256, 0, st>>>(t, didx + b0, B, d.out, bt);
            gather_rows_kernel<<<g2, 256, 0, st>>>(mask, didx + b0, B, d.out, bm);
            ndconv_count_launch();
            ndconv_count_launch();
            ndconv_count_launch();
            if ((s = grad_into(net, bx, bt, bm, B, net->grad, dloss, st))) break;
            net->step++;
            const double c1 = 1.0 - std::pow((double)b1, (double)net->step);
            const double c2 = 1.0 - std::pow((double)b2, (double)net->step);
            const float lr_t = (float)(lr * std::sqrt(c2) / c1);
            adam_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, st>>>(net->P, net->grad, net->m1, net->m2, cnt,
                                                                        lr_t, b1, b2, eps);
            ndconv_count_launch();
        }
        // the per-epoch copy reuses the host index array: finish before reshuffling
        cudaStreamSynchronize(st);
    }
    if (s == NDCONV_OK && final_loss) {
        // loss over the whole set with the final parameters
        s = grad_into(net, x, t, mask, n, net->grad, dloss, st);
        if (s == NDCONV_OK) cudaMemcpyAsync(final_loss, dloss, sizeof(float), cudaMemcpyDeviceToHost, st);
    }
    cudaStreamSynchronize(st);
    e = cudaGetLastError();
    cudaFree(bx);
    cudaFree(didx);
    if (s) return s;
    if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
    return NDCONV_OK;
}
