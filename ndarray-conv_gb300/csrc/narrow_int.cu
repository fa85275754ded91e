// 8- and 16-bit integer direct convolution (ConvExt::conv for u8 / i8 / u16
// / i16, src/conv/mod.rs:128-200, wrapping arithmetic as release-mode Rust).
//
// The data and the kernel are widened to 32 bits on the device (one pass
// each, honouring the callers' strides), summed by the 32-bit direct
// kernels, and the 32-bit results are truncated into the caller's output.
// A wrapping sum of products modulo 2^32 keeps the low 8 or 16 bits of the
// same sum modulo 2^8 or 2^16, and those depend only on the low bits of the
// terms, so the truncated result is the element type's own wrapping sum
// whether the values were sign- or zero-extended.  Border constants reach
// the 32-bit plan as the same integer values.
#include "common.cuh"
#include "direct.h"
#include "geometry.h"

namespace ndconv {
namespace {

template <typename S>
__global__ void widen_kernel(const S *__restrict__ x, int64_t n0, int64_t n1, int64_t n2, int64_t s0, int64_t s1,
                             int64_t s2, int32_t *__restrict__ out) {
    const int64_t total = n0 * n1 * n2;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total;
         u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i2 = u % n2, r = u / n2;
        const int64_t i1 = r % n1, i0 = r / n1;
        out[u] = (int32_t)x[i0 * s0 + i1 * s1 + i2 * s2];
    }
}

// low bits of each 32-bit sum (conversion through the unsigned type is the
// defined modulo reduction)
template <typename U>
__global__ void narrow_kernel(const int32_t *__restrict__ y, int64_t n, U *__restrict__ out) {
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x)
        out[u] = (U)(uint32_t)y[u];
}

unsigned grid_for(int64_t n) {
    const int64_t b = (n + 255) / 256;
    return (unsigned)(b < 152 * 16 ? (b < 1 ? 1 : b) : 152 * 16);
}

template <typename S, typename U>
int run_narrow(const Plan3 &P, const void *data, const void *kernel, void *out, cudaStream_t st) {
    const AxisGeom *A = P.ax;
    const int64_t nx = A[0].n * A[1].n * A[2].n, nk = A[0].K * A[1].K * A[2].K;
    const int64_t ny = A[0].out * A[1].out * A[2].out;
    int32_t *buf = nullptr;
    NDCONV_CUDA_OK(cudaMallocAsync((void **)&buf, sizeof(int32_t) * (size_t)(nx + nk + ny), st));
    int32_t *x32 = buf, *k32 = buf + nx, *y32 = buf + nx + nk;
    widen_kernel<S><<<grid_for(nx), 256, 0, st>>>(static_cast<const S *>(data), A[0].n, A[1].n, A[2].n, A[0].xs,
                                                   A[1].xs, A[2].xs, x32);
    widen_kernel<S><<<grid_for(nk), 256, 0, st>>>(static_cast<const S *>(kernel), A[0].K, A[1].K, A[2].K, A[0].ks,
                                                   A[1].ks, A[2].ks, k32);
    ndconv_count_launch(2);
    // the same problem over contiguous 32-bit copies
    Plan3 Q = P;
    Q.dtype = NDCONV_I32;
    Q.ax[2].xs = 1;
    Q.ax[1].xs = A[2].n;
    Q.ax[0].xs = A[1].n * A[2].n;
    Q.ax[2].ks = 1;
    Q.ax[1].ks = A[2].K;
    Q.ax[0].ks = A[1].K * A[2].K;
    cudaError_t e = direct_conv_launch<int32_t>(x32, k32, y32, Q.direct<int32_t>(), st, 0);
    if (e == cudaSuccess) {
        narrow_kernel<U><<<grid_for(ny), 256, 0, st>>>(y32, ny, static_cast<U *>(out));
        ndconv_count_launch();
        e = cudaGetLastError();
    }
    cudaFreeAsync(buf, st);  // stream-ordered: after the launches have finished with it
    if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
    return NDCONV_OK;
}

}  // namespace

int conv_narrow_int(const Plan3 &P, const void *data, const void *kernel, void *out, cudaStream_t st) {
    switch (P.dtype) {
    case NDCONV_U8: return run_narrow<uint8_t, uint8_t>(P, data, kernel, out, st);
    case NDCONV_I8: return run_narrow<int8_t, uint8_t>(P, data, kernel, out, st);
    case NDCONV_U16: return run_narrow<uint16_t, uint16_t>(P, data, kernel, out, st);
    case NDCONV_I16: return run_narrow<int16_t, uint16_t>(P, data, kernel, out, st);
    default: return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "not an 8- or 16-bit integer element type");
    }
}

}  // namespace ndconv
