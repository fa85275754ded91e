// ndconv_conv_fft_noalloc: the FFT convolution for callers that cannot
// allocate device memory.
//
// Some callers cannot call cudaMalloc at all: real-time or embedded hosts
// that forbid allocation after start-up (an allocation can block or fail at
// an arbitrary time), and plugins whose host application owns every device
// allocation.  This entry point runs the same kernels as
// ndconv_conv_fft but takes its spectrum buffers and twiddle tables from a
// fixed, file-scope device array instead of allocating them.  The array
// (kNoAllocScratchBytes = 16 MiB) is part of the library image: every GPU
// on which the library is loaded holds it until the process exits.
#include <mutex>

#include "common.cuh"
#include "fft.h"
#include "geometry.h"

namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)16 << 20;

// The scratch itself.  In host code this name is a host-side stand-in for
// the symbol, not a device address: the address a kernel may use comes from
// cudaGetSymbolAddress (below), once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the scratch on the current device, looked up on the
// first call made with that device current.
int scratch_for_current_device(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return ndconv_fail(NDCONV_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress((void **)&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
        g_scratch_addr[dev] = ptr;
    }
    *out = g_scratch_addr[dev];
    return NDCONV_OK;
}

template <typename T>
int run(const ndconv::Plan3 &P, const void *data, const void *kernel, void *out, cudaStream_t st) {
    using namespace ndconv;
    const Geom3<T> g = P.geom<T>();
    const size_t spectra = (conv_fft_scratch_bytes<T>(g) + 255) / 256 * 256;
    if (spectra >= kNoAllocScratchBytes)
        return ndconv_fail(NDCONV_ERR_NO_MEMORY,
                           "problem needs more than the 16 MiB scratch of ndconv_conv_fft_noalloc");
    void *base = nullptr;
    int s = scratch_for_current_device(&base);
    if (s) return s;
    // spectra first, twiddle tables after them in the same array
    TwArena arena{};
    arena.base = static_cast<unsigned char *>(base) + spectra;
    arena.cap = kNoAllocScratchBytes - spectra;
    arena.used = 0;
    arena.st = st;
    TwArenaScope scope(&arena);
    return conv_fft_run<T>(g, P.reverse, static_cast<const T *>(data), static_cast<const T *>(kernel),
                           static_cast<T *>(out), nullptr, st, base, spectra);
}

}  // namespace

// See include/ndconv.h.  Allocates nothing: no cudaMalloc, cudaFree or
// allocating library call on any path.  The first call on a device looks up
// the scratch address (cudaGetSymbolAddress); make that first call before
// any stream capture.  All calls share the one scratch array and it keeps
// the previous call's contents; every location a call reads was written
// earlier in the same call, so nothing needs clearing.  Calls whose GPU work
// overlaps (different streams, or several host threads) race on the scratch
// and must be serialised by the caller.
extern "C" int ndconv_conv_fft_noalloc(const ndconv_problem *p, const void *data, const void *kernel,
                                       void *out, void *stream) {
    ndconv::Plan3 P;
    int s = ndconv::plan_problem(p, 1, &P);
    if (s) return s;
    if (!data || !kernel || !out) return ndconv_fail(NDCONV_ERR_INVALID, "null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    switch (P.dtype) {
    case NDCONV_F32: return run<float>(P, data, kernel, out, st);
    case NDCONV_F64: return run<double>(P, data, kernel, out, st);
    case NDCONV_C32: return run<c32>(P, data, kernel, out, st);
    case NDCONV_C64: return run<c64>(P, data, kernel, out, st);
    default:
        return ndconv_fail(NDCONV_ERR_UNSUPPORTED,
                           "integer FFT convolution is not supported (documented broken upstream)");
    }
}
