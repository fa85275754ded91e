// Batched convolution of instances held in host memory: the library stages
// chunks of instances through its own device buffers so that host->device
// copies, the convolution and device->host copies of successive chunks
// overlap (three streams, a ring of slots).  No reference counterpart: the
// crate works on host arrays one call at a time.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <vector>

#include "common.cuh"
#include "direct.h"
#include "fft.h"
#include "geometry.h"
#include "ndconv.h"

using namespace ndconv;

namespace {
size_t elem_size(int dtype) {
    switch (dtype) {
    case NDCONV_F32: return 4;
    case NDCONV_I32: return 4;
    case NDCONV_F64: return 8;
    case NDCONV_C32: return 8;
    default: return 16;
    }
}

template <typename T>
int run_chunk(const Plan3 &P, int algo, int64_t cnt, const void *const *dx, const void *const *dk, void *const *dy,
              ndconv_fft_processor *proc, cudaStream_t st) {
    if (algo == NDCONV_ALGO_DIRECT) {
        cudaError_t e = direct_conv_batch_launch<T>(cnt, (const T *const *)dx, (const T *const *)dk, (T *const *)dy,
                                                    P.direct<T>(), st);
        if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
        return NDCONV_OK;
    }
    if constexpr (std::is_same<T, int32_t>::value) {
        return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "integer FFT convolution is not supported");
    } else {
        return conv_fft_batch_run<T>(P.geom<T>(), P.reverse, cnt, (const T *const *)dx, (const T *const *)dk,
                                     (T *const *)dy, proc, st);
    }
}
}  // namespace

extern "C" int ndconv_conv_batch_host(const ndconv_problem *p, int32_t algo, int64_t n, const void *const *data,
                                      const void *const *kernel, void *const *out, ndconv_fft_processor *proc,
                                      void *stream) {
    if (algo != NDCONV_ALGO_DIRECT && algo != NDCONV_ALGO_FFT)
        return ndconv_fail(NDCONV_ERR_INVALID, "algo must be 0 (direct) or 1 (FFT)");
    Plan3 P;
    int s = plan_problem(p, algo, &P);
    if (s) return s;
    if (single_call_int(P.dtype))
        return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "this integer element type runs ndconv_conv only");
    if (n < 0) return ndconv_fail(NDCONV_ERR_INVALID, "negative batch size");
    if (n == 0) return NDCONV_OK;
    if (!data || !kernel || !out) return ndconv_fail(NDCONV_ERR_INVALID, "null pointer array");
    for (int a = 0; a < 3; a++)
        if (p->data_strides[a] != 0 || p->kernel_strides[a] != 0)
            return ndconv_fail(NDCONV_ERR_INVALID, "host batches take contiguous arrays");
    const size_t es = elem_size(P.dtype);
    const AxisGeom *A = P.ax;
    const size_t bx = es * (size_t)(A[0].n * A[1].n * A[2].n), bk = es * (size_t)(A[0].K * A[1].K * A[2].K);
    const size_t by = es * (size_t)(A[0].out * A[1].out * A[2].out);
    const size_t per = (bx + bk + by + 255) / 256 * 256 + 256;
    // chunks of ~chunk_mb MB of inputs and outputs (at least one instance) in
    // a ring of NS slots: both copy directions stream concurrently (the link
    // carries ~210 GB/s one way, ~340 GB/s both ways on a GB300), and a ring
    // deeper than two keeps a chunk's output copy from holding up the next
    // convolution.  NDCONV_HOST_CHUNK_MB / NDCONV_HOST_SLOTS override.
    size_t chunk_mb = 16;
    int NS = 3;
    if (const char *v = std::getenv("NDCONV_HOST_CHUNK_MB")) chunk_mb = std::max<long>(1, std::atol(v));
    if (const char *v = std::getenv("NDCONV_HOST_SLOTS")) NS = (int)std::min<long>(8, std::max<long>(2, std::atol(v)));
    int64_t C = (int64_t)((chunk_mb << 20) / (bx + by + 1));
    C = std::max<int64_t>(1, std::min<int64_t>(C, n));
    const int64_t n_chunks = (n + C - 1) / C;
    if (n_chunks < NS) NS = (int)std::max<int64_t>(1, n_chunks);
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char *buf = nullptr;
    NDCONV_CUDA_OK(cudaMallocAsync((void **)&buf, NS * (size_t)C * per + NS * 3 * sizeof(void *) * (size_t)C, st));
    // device pointer arrays of all slots, written once
    std::vector<void *> ptrs((size_t)(NS * 3 * C));
    for (int slot = 0; slot < NS; slot++)
        for (int64_t i = 0; i < C; i++) {
            unsigned char *b = buf + ((size_t)slot * C + i) * per;
            ptrs[(size_t)((slot * 3 + 0) * C + i)] = b;
            ptrs[(size_t)((slot * 3 + 1) * C + i)] = b + (bx + 255) / 256 * 256;
            ptrs[(size_t)((slot * 3 + 2) * C + i)] = b + (bx + 255) / 256 * 256 + (bk + 255) / 256 * 256;
        }
    void **dptr = reinterpret_cast<void **>(buf + NS * (size_t)C * per);
    cudaError_t e = cudaMemcpyAsync(dptr, ptrs.data(), sizeof(void *) * ptrs.size(), cudaMemcpyHostToDevice, st);
    cudaStream_t sin = nullptr, sout = nullptr;
    // per slot: inputs landed, convolution done, outputs copied
    std::vector<cudaEvent_t> evs((size_t)(3 * NS), nullptr);
    auto ev = [&](int slot, int j) -> cudaEvent_t & { return evs[(size_t)(slot * 3 + j)]; };
    bool made = false;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sin, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sout, cudaStreamNonBlocking);
    for (size_t j = 0; j < evs.size() && e == cudaSuccess; j++) e = cudaEventCreateWithFlags(&evs[j], cudaEventDisableTiming);
    made = (e == cudaSuccess);
    cudaEvent_t start = nullptr;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&start, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(start, st);  // the pointer upload and allocation come first
    if (e == cudaSuccess) e = cudaStreamWaitEvent(sin, start, 0);
    s = (e == cudaSuccess) ? NDCONV_OK : ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
    // every enqueue call is checked; the first failure ends the loop (what
    // was enqueued still completes before the buffer is released below)
    auto chk = [&](cudaError_t r) {
        if (r != cudaSuccess && s == NDCONV_OK) s = ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(r));
    };
    for (int64_t c0 = 0, chunk = 0; c0 < n && s == NDCONV_OK; c0 += C, chunk++) {
        const int slot = (int)(chunk % NS);
        const int64_t cnt = std::min<int64_t>(C, n - c0);
        // inputs: the slot's inputs are free once its previous convolution is done
        if (chunk >= NS) chk(cudaStreamWaitEvent(sin, ev(slot, 1), 0));
        for (int64_t i = 0; i < cnt && s == NDCONV_OK; i++) {
            chk(cudaMemcpyAsync(ptrs[(size_t)((slot * 3 + 0) * C + i)], data[c0 + i], bx, cudaMemcpyHostToDevice, sin));
            chk(cudaMemcpyAsync(ptrs[(size_t)((slot * 3 + 1) * C + i)], kernel[c0 + i], bk, cudaMemcpyHostToDevice, sin));
        }
        chk(cudaEventRecord(ev(slot, 0), sin));
        // convolution: after the inputs and after the slot's previous outputs left
        chk(cudaStreamWaitEvent(st, ev(slot, 0), 0));
        if (chunk >= NS) chk(cudaStreamWaitEvent(st, ev(slot, 2), 0));
        if (s) break;
        const void *const *dx = (const void *const *)(dptr + (slot * 3 + 0) * C);
        const void *const *dk = (const void *const *)(dptr + (slot * 3 + 1) * C);
        void *const *dy = (void *const *)(dptr + (slot * 3 + 2) * C);
        switch (P.dtype) {
        case NDCONV_F32: s = run_chunk<float>(P, algo, cnt, dx, dk, dy, proc, st); break;
        case NDCONV_F64: s = run_chunk<double>(P, algo, cnt, dx, dk, dy, proc, st); break;
        case NDCONV_I32: s = run_chunk<int32_t>(P, algo, cnt, dx, dk, dy, proc, st); break;
        case NDCONV_C32: s = run_chunk<c32>(P, algo, cnt, dx, dk, dy, proc, st); break;
        default: s = run_chunk<c64>(P, algo, cnt, dx, dk, dy, proc, st); break;
        }
        chk(cudaEventRecord(ev(slot, 1), st));
        // outputs back to the host
        chk(cudaStreamWaitEvent(sout, ev(slot, 1), 0));
        for (int64_t i = 0; i < cnt && s == NDCONV_OK; i++)
            chk(cudaMemcpyAsync(out[c0 + i], ptrs[(size_t)((slot * 3 + 2) * C + i)], by, cudaMemcpyDeviceToHost, sout));
        chk(cudaEventRecord(ev(slot, 2), sout));
    }
    // the caller's stream covers everything: wait for the last copies, then free
    if (made) {
        for (int slot = 0; slot < NS; slot++) cudaStreamWaitEvent(st, ev(slot, 2), 0);
    }
    cudaFreeAsync(buf, st);
    for (cudaEvent_t x : evs)
        if (x) cudaEventDestroy(x);
    if (start) cudaEventDestroy(start);
    if (sin) cudaStreamDestroy(sin);
    if (sout) cudaStreamDestroy(sout);
    if (s) return s;
    e = cudaGetLastError();
    if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
    return NDCONV_OK;
}
