// FFT plans and twiddle tables: radix factorisation (make_plan), transform
// lengths (smooth_size / pow2_size) and the per-device cache of twiddle
// tables generated in FP64 on the GPU.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "fft.h"
#include "fft_core.cuh"

namespace ndconv {

// ------------------------------------------------------------- twiddles --
template <typename C>
__global__ void gen_twiddles_kernel(C *tw, int L) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < L; t += gridDim.x * blockDim.x) {
        double s, c;
        sincospi(-2.0 * (double)t / (double)L, &s, &c);  // exp(-2 pi i t / L) in FP64
        tw[t].re = (decltype(tw[t].re))c;
        tw[t].im = (decltype(tw[t].im))s;
    }
}

// Stage table of a plan (FftPlanDev::tws): entry e of stage s is
// w^(t r), w = exp(-2 pi i / (Ns R)), t = (e - twoff[s]) / R, r its
// remainder; the exponent t r is reduced mod Ns R before the FP64 sincospi.
// Entries between stages (even alignment) are set to 1.
template <typename C>
__global__ void gen_stage_twiddles_kernel(C *tw, const __grid_constant__ FftPlanDev pl) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < pl.twn; e += gridDim.x * blockDim.x) {
        double s = 0, c = 1;
        for (int st = 1; st < pl.nst; st++) {
            const int R = pl.rad[st];
            const int64_t nsr = (int64_t)pl.ns[st].d * R;
            const int64_t o = e - pl.twoff[st];
            if (o >= 0 && o < nsr) {
                const int64_t m = ((o / R) * (o % R)) % nsr;
                sincospi(-2.0 * (double)m / (double)nsr, &s, &c);
                break;
            }
        }
        tw[e].re = (decltype(tw[e].re))c;
        tw[e].im = (decltype(tw[e].im))s;
    }
}

thread_local TwArena *g_tw_arena = nullptr;

TwArenaScope::TwArenaScope(TwArena *a) : prev(g_tw_arena) { g_tw_arena = a; }
TwArenaScope::~TwArenaScope() { g_tw_arena = prev; }

namespace {
std::mutex g_tw_mu;
// (device, bytes-per-complex, L, kind) -> table; kind 0: tw[t] = exp(-2 pi i t / L),
// kind 1: the stage table of make_plan(L)
std::map<std::tuple<int, int, int, int>, void *> g_tw;

// entries of a table of kind `kind` for length L (pl: make_plan(L) for kind 1)
size_t tw_entries(int L, int kind, const FftPlanDev *pl) {
    const int n = kind ? pl->twn : L;
    return (size_t)(n > 0 ? n : 1);
}

template <typename C> void launch_gen_twiddles(C *p, int L, int kind, const FftPlanDev *pl, cudaStream_t st) {
    const size_t n = tw_entries(L, kind, pl);
    int blocks = (int)((n + 255) / 256);
    if (blocks > 1024) blocks = 1024;
    if (blocks < 1) blocks = 1;
    if (kind) gen_stage_twiddles_kernel<C><<<blocks, 256, 0, st>>>(p, *pl);
    else gen_twiddles_kernel<C><<<blocks, 256, 0, st>>>(p, L);
    ndconv_count_launch();
}

// Tables carved from a caller-provided arena and generated on its stream
// (no allocation, no synchronisation).
template <typename C> int arena_twiddles(TwArena *a, int L, int kind, const FftPlanDev *pl, const C **out) {
    for (int i = 0; i < a->n; i++)
        if (a->len[i] == L && a->elem[i] == (int)sizeof(C) && a->kind[i] == kind) {
            *out = (const C *)a->table[i];
            return NDCONV_OK;
        }
    const size_t off = (a->used + 255) / 256 * 256;
    const size_t bytes = sizeof(C) * tw_entries(L, kind, pl);
    if (a->n >= TwArena::kMaxTables || off + bytes > a->cap)
        return ndconv_fail(NDCONV_ERR_NO_MEMORY, "twiddle tables do not fit the provided scratch");
    C *p = reinterpret_cast<C *>(a->base + off);
    launch_gen_twiddles<C>(p, L, kind, pl, a->st);
    NDCONV_CUDA_OK(cudaGetLastError());
    a->used = off + bytes;
    a->len[a->n] = L;
    a->elem[a->n] = (int)sizeof(C);
    a->kind[a->n] = kind;
    a->table[a->n] = p;
    a->n++;
    *out = p;
    return NDCONV_OK;
}

}  // namespace

// kind 0: tw[t] = exp(-2 pi i t / L); kind 1: the stage table of *pl
template <typename C> int get_twiddles(int L, const C **out, int kind, const FftPlanDev *pl) {
    if (g_tw_arena) return arena_twiddles<C>(g_tw_arena, L, kind, pl, out);
    int dev = 0;
    NDCONV_CUDA_OK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_tw_mu);
    auto key = std::make_tuple(dev, (int)sizeof(C), L, kind);
    auto it = g_tw.find(key);
    if (it != g_tw.end()) {
        *out = (const C *)it->second;
        return NDCONV_OK;
    }
    void *p = nullptr;
    NDCONV_CUDA_OK(cudaMalloc(&p, sizeof(C) * tw_entries(L, kind, pl)));
    cudaStream_t s;
    NDCONV_CUDA_OK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    launch_gen_twiddles<C>((C *)p, L, kind, pl, s);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (e != cudaSuccess) {
        cudaFree(p);
        return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
    }
    g_tw[key] = p;
    *out = (const C *)p;
    return NDCONV_OK;
}
template int get_twiddles<c32>(int, const c32 **, int, const FftPlanDev *);
template int get_twiddles<c64>(int, const c64 **, int, const FftPlanDev *);

// Radix factorisation: 8s, 4, 2, 3s, 5s, then other primes (generic
// butterfly up to kMaxGenericRadix).  Returns false if a prime factor is
// larger than that.
// Radices: 16s for the power of two (one radix-10 stage takes a factor 2
// with a factor 5, then 8 / 4 / 2 for the rest), then odd factors.  Fewer,
// wider stages mean fewer shared-memory round trips and barriers.
bool make_plan(int L, FftPlanDev &pl) {
    pl.L = L;
    pl.nst = 0;
    int r = L;
    const bool ten = (r % 10 == 0) && (r % 4 != 0 || r % 32 == 0);
    if (ten) r /= 10;
    while (r % 16 == 0) { pl.rad[pl.nst++] = 16; r /= 16; }
    if (r % 8 == 0) { pl.rad[pl.nst++] = 8; r /= 8; }
    if (r % 4 == 0) { pl.rad[pl.nst++] = 4; r /= 4; }
    if (r % 2 == 0) { pl.rad[pl.nst++] = 2; r /= 2; }
    if (ten) pl.rad[pl.nst++] = 10;
    for (int f = 3; r > 1; f += 2) {
        while (r % f == 0) {
            if (f > kMaxGenericRadix || pl.nst >= kMaxStages) return false;
            pl.rad[pl.nst++] = f;
            r /= f;
        }
        if ((int64_t)f * f > r && r > 1) {
            if (r > kMaxGenericRadix || pl.nst >= kMaxStages) return false;
            pl.rad[pl.nst++] = r;
            r = 1;
        }
    }
    uint32_t ns = 1;
    int off = 0;
    for (int s = 0; s < pl.nst; s++) {
        pl.ns[s] = make_fastdiv(ns);
        pl.twoff[s] = 0;
        if (s > 0) {
            off = (off + 1) & ~1;
            pl.twoff[s] = off;
            off += (int)ns * pl.rad[s];
        }
        ns *= (uint32_t)pl.rad[s];
    }
    pl.twn = off;
    pl.tws = nullptr;
    return true;
}

// Relative cost of one Stockham stage per element, by radix (each stage is
// one shared-memory round trip; larger radices do more arithmetic).
double stage_cost(int r) {
    switch (r) {
    case 16: return 1.25;
    case 10: return 1.2;
    case 8: return 1.0;
    case 4: return 0.75;
    case 2: return 0.6;
    case 3: return 0.8;
    case 5: return 1.0;
    case 7: return 1.3;
    default: return 4.0;
    }
}

// Cheapest 2^a 3^b 5^c 7^d >= n (even when asked; the real axis transforms
// half of it), among sizes up to 1.35 n.
int64_t smooth_size(int64_t n, bool even) {
    if (n <= 1) return even ? 2 : 1;
    int64_t best = INT64_MAX;
    double best_cost = 1e300;
    const int64_t lim = n + n * 35 / 100 + 8;
    for (int64_t p7 = 1; p7 <= 4 * lim; p7 *= 7)
        for (int64_t p5 = p7; p5 <= 4 * lim; p5 *= 5)
            for (int64_t p3 = p5; p3 <= 4 * lim; p3 *= 3) {
                int64_t v = p3;
                while (v < n || (even && (v & 1))) v *= 2;
                if (v > lim && best != INT64_MAX) continue;
                FftPlanDev pl;
                const int64_t L = even ? v / 2 : v;
                double c = 1e300;
                if (L < (1 << 30) && make_plan((int)L, pl)) {
                    c = 0;
                    for (int s = 0; s < pl.nst; s++) c += stage_cost(pl.rad[s]);
                    c *= (double)L;
                }
                if (c < best_cost || (c == best_cost && v < best)) {
                    best_cost = c;
                    best = v;
                }
            }
    return best;
}

int64_t pow2_size(int64_t n, bool even) {
    int64_t v = even ? 2 : 1;
    while (v < n) v *= 2;
    return v;
}

}  // namespace ndconv
