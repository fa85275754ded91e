// Direct convolution on the 5th-generation tensor cores with 3xBF16 split
// products (f32 data and kernels, f32 accumulation in tensor memory).
//
// Each f32 value v is split as hi = bf16(v), lo = bf16(v - hi), and a
// product x k is formed as xh kh + xh kl + xl kh (the dropped xl kl term and
// the splits' rounding leave ~2^-16 relative error per product, below the
// 1e-5 normwise bar).
//
// Lowering: row correlations on the tensor cores, shifted sums in the
// epilogue.  For an output plane oz and a tile of BN output columns starting
// at ox0, correlating padded data row r with kernel row ky gives
//   P[r][ky][b] = sum over kz, tx of kf[kz][ky][tx] X[oz s0 + kz d0][r][(ox0 + b) s2 + tx d2]
// and output row oy is sum over ky of P[oy s1 + ky d1][ky][b].  The first sum
// is one GEMM per 64-wide K chunk:
//   D[m][n] = sum_c X[r0 + m][ox0 s2 + c] T[n][c],    n = (ky, b)
// with M = 128 consecutive padded rows (TMEM lanes), N = G BN (G kernel rows
// of a group times BN output columns: TMEM columns), K = the tile's input
// window (BN - 1) s2 + (K2 - 1) d2 + 1 rounded up to 16, and T the Toeplitz
// bands of the group's kernel rows: T[(ky, b)][c] = kf[kz][ky][tx] where
// c = b s2 + tx d2.  The data operand (a 128-row x 64-column TMA box of the
// padded plane) is shared by the G kernel rows, so one MMA covers a whole
// group; the plane taps kz accumulate in TMEM.  The epilogue moves D through
// shared memory and sums each output over the group's kernel rows; kernels
// with more than G rows run as several groups whose sums add in registers.
// A tile keeps the output rows whose G input rows lie inside its 128 rows.
//
// Operands are K-major bf16 tiles of 64 elements per row (one 128-byte
// swizzled row) staged by TMA from two pre-built planes in global memory:
// the padded data (border map applied once, split into hi / lo) and the
// Toeplitz bands.  The kernel is persistent (one CTA per SM over contiguous
// tile ranges; batches of instances of one geometry share the launch) and
// warp-specialised: one thread issues TMA, one issues tcgen05.mma into two
// TMEM accumulators in turn, eight warps drain the other with tcgen05.ld.
// Every mbarrier wait is bounded; a timeout (not expected) writes NaN to the
// CTA's tiles, records the event in a library-owned per-device word (read
// and cleared by ndconv_bf16x3_status), waits (bounded) for the TMA loads and
// MMAs already in flight, and the CTA still releases TMEM.
// Non-finite inputs (flagged per block by the pre-pass) make every CTA compute
// its tiles with the FP32 direct loop instead, like the reference's sums.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "direct.h"
#include "direct_blocks.cuh"
#include "geometry.h"
#include "ndconv.h"

namespace ndconv {
namespace bf16x3 {

constexpr int BM = 128;                 // padded rows per tile (TMEM lanes)
constexpr int KC = 64;                  // bf16 per K chunk: one 128-byte swizzled row
constexpr int A_BYTES = BM * KC * 2;    // one data box (hi or lo)
constexpr int RP = 20;                  // floats per row of the epilogue's row block (16 + 4: no bank conflicts)
constexpr int kRowBlockBytes = 3 * BM * RP * 4;  // the epilogue's exchange / row blocks
constexpr int kMaxStages = 4;
constexpr int kSmemLimit = 227 * 1024;
constexpr int kSmemExtra = 1024 + 256 + kRowBlockBytes;  // alignment slack, barriers, row block
constexpr long long kWaitCycles = 2000000000LL;  // ~1 s of polling before a wait gives up
constexpr int kThreads = 320;  // warps 0-7 epilogue (two groups), 8 TMA producer, 9 MMA issuer

// Timeouts of any launch on this device since the last ndconv_bf16x3_status
// call (a file-scope device variable: one per device that loads the library).
__device__ int g_timeouts;

struct Params {
    int64_t out0, out1, out2;
    int64_t s0, d0, s1, d1, s2;
    int K0;
    int G, ngroups;      // kernel rows per group (zero rows pad the last), groups
    int N;               // G * BN: MMA N and Toeplitz rows per (kz, group)
    int mvalid;          // output rows per tile
    int64_t nrt, nct;    // tiles along the middle and contiguous axes
    int64_t ntiles;      // out0 * nrt * nct
    int nchunk, klast;   // 64-wide K chunks per (group, kz); 16-wide steps in the last one
    int stages, stage_bytes, ring_bytes;  // ring_bytes includes the resident Toeplitz tiles
    int bres, b_off;     // Toeplitz tiles of all groups resident (at byte b_off), or in each stage
    int tmem_cols;
    int shfl_epi;        // epilogue by warp shuffles (unit middle stride, (G - 1) d1 < 32)
    int row_epi;         // one kernel row per group and unit middle stride: TMEM row m is output row m
    uint32_t idesc;
    float *y;
    int64_t ys0, ys1;
    int64_t xlast;     // outputs in the last output row (a folded row's ragged end; out2 otherwise)
    const int *flags;  // per pre-pass block: a non-finite input seen (any instance)
    int nflags;
    DirectParams<float> dp;  // FP32 fallback
    const float *x, *k;
    // batches of instances sharing the geometry: device arrays of their
    // pointers (null for one instance: x, k, y above); tiles per instance,
    // padded planes per instance (plane index of instance i: i P0 + ...),
    // Toeplitz rows per instance
    const float *const *xs;
    const float *const *ks;
    float *const *ys;
    int64_t tiles_inst, P0, Rt;
};

// ---- PTX wrappers --------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
                 : "memory");
}
// bounded wait for the phase of the given parity; false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity) {
    const uint32_t a = smem_u32(b);
    const long long t0 = clock64();
    for (;;) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
        if (clock64() - t0 > kWaitCycles) return false;
    }
}
__device__ __forceinline__ void tma_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
// K-major operand in the 128-byte swizzle layout: rows of 128 B, 8-row
// groups 1024 B apart (SBO), descriptor version 1, layout type 2 (128B).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)1 << 16;             // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
    d |= (uint64_t)1 << 46;             // descriptor version
    d |= (uint64_t)2 << 61;             // 128-byte swizzle
    return d;
}
// kind::f16 instruction descriptor: D f32, A/B bf16, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        ::"r"(tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t addr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(addr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// tcgen05.ld without the wait, and the wait tied to the loaded registers (so
// that no use of them is scheduled before it)
__device__ __forceinline__ void tmem_ld16_issue(uint32_t addr, uint32_t *r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(addr));
}
__device__ __forceinline__ void tmem_ld_wait(uint32_t *r) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15])
                 :
                 : "memory");
}

// ---- pre-passes -----------------------------------------------------------
// Padded data planes [n][rows][W] (hi, lo) of n instances (xs: device
// array of their data pointers, or null for the one instance x); zero beyond
// column lim.  Unfolded (hop 0): rows = P0 P1 planes' rows, lim the padded
// extent.  A folded row (hop > 0): row r holds padded positions r hop ..
// r hop + lim - 1 of the one padded row.  A thread converts 8 consecutive
// samples of a row and stores them as 16-byte vectors (W is a multiple of 8).
// (blocks bid of nblk of the pre-pass launch; returns whether this thread saw
// a non-finite value)
__device__ __forceinline__ bool split_part(const float *__restrict__ x, const float *const *xs, int64_t n,
                                           const Geom3<float> &g, int64_t W, int64_t rows, int64_t hop,
                                           int64_t lim, __nv_bfloat16 *__restrict__ hi,
                                           __nv_bfloat16 *__restrict__ lo, int64_t bid, int64_t nblk) {
    const AxisGeom &A2 = g.ax[2];
    const int64_t cw = W / 8, total = n * rows * cw;
    bool bad = false;
    for (int64_t u = bid * blockDim.x + threadIdx.x; u < total; u += nblk * blockDim.x) {
        const int64_t grow = u / cw, c0 = (u - grow * cw) * 8;  // row over all instances
        const int64_t inst = grow / rows, row = grow - inst * rows;
        const float *xi = xs ? xs[inst] : x;
        int64_t m0 = 0, m1 = 0, q0 = c0;  // q0: padded position of the first sample
        if (hop) {
            q0 += row * hop;
        } else {
            m0 = axis_map(g.ax[0], row / g.ax[1].L);
            m1 = axis_map(g.ax[1], row % g.ax[1].L);
        }
        float v[8];
        const int64_t j0 = q0 - A2.p0;  // input index of the first sample
        if (m0 >= 0 && m1 >= 0 && A2.xs == 1 && j0 >= 0 && j0 + 8 <= A2.n && c0 + 8 <= lim) {
            // interior samples of a contiguous row: plain (vector) loads
            const float *src = xi + m0 * g.ax[0].xs + m1 * g.ax[1].xs + j0;
            if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
                const float4 a = __ldg(reinterpret_cast<const float4 *>(src));
                const float4 b = __ldg(reinterpret_cast<const float4 *>(src) + 1);
                v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
                v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
            } else if ((reinterpret_cast<uintptr_t>(src) & 7) == 0) {
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float2 a = __ldg(reinterpret_cast<const float2 *>(src) + q);
                    v[2 * q] = a.x;
                    v[2 * q + 1] = a.y;
                }
            } else {
#pragma unroll
                for (int q = 0; q < 8; q++) v[q] = __ldg(src + q);
            }
        } else {
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int64_t i2 = q0 + q;
                v[q] = c0 + q < lim && i2 < A2.L ? resolve_padded<float>(xi, g, m0, m1, axis_map(A2, i2)) : 0.f;
            }
        }
        uint32_t h[4], l[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            if (!isfinite(v[2 * e]) || !isfinite(v[2 * e + 1])) bad = true;
            const __nv_bfloat162 hh = __floats2bfloat162_rn(v[2 * e], v[2 * e + 1]);
            const float2 hf = __bfloat1622float2(hh);
            const __nv_bfloat162 ll = __floats2bfloat162_rn(v[2 * e] - hf.x, v[2 * e + 1] - hf.y);
            h[e] = *reinterpret_cast<const uint32_t *>(&hh);
            l[e] = *reinterpret_cast<const uint32_t *>(&ll);
        }
        *reinterpret_cast<uint4 *>(hi + grow * W + c0) = make_uint4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<uint4 *>(lo + grow * W + c0) = make_uint4(l[0], l[1], l[2], l[3]);
    }
    return bad;
}

// Toeplitz bands [n][K0][ngroups][G][BN][Cp] (hi, lo): row (kz, group, kl, b)
// of an instance, column c holds kf[kz][ky][tx] when ky = group G + kl < K1
// and c = b s2 + tx d2 (kf: the kernel in tap order, reversed for
// convolution); zero elsewhere (the padding rows of the last group included).
// One warp per band row (its coordinates decoded once), lanes along c.
__device__ __forceinline__ bool toeplitz_part(const float *__restrict__ k1, const float *const *ks, int64_t n,
                                              const Geom3<float> &g, int reverse, int G, int BN, int ngroups,
                                              int64_t Cp, __nv_bfloat16 *__restrict__ hi,
                                              __nv_bfloat16 *__restrict__ lo, int64_t bid, int64_t nblk) {
    const AxisGeom &A0 = g.ax[0], &A1 = g.ax[1], &A2 = g.ax[2];
    const int64_t per = A0.K * ngroups * G * BN, rows = n * per;
    const int lane = threadIdx.x & 31;
    const int64_t wstep = nblk * (blockDim.x >> 5);
    bool bad = false;
    for (int64_t row = bid * (blockDim.x >> 5) + (threadIdx.x >> 5); row < rows; row += wstep) {
        const int64_t inst = row / per;
        int64_t r = row - inst * per;
        const int64_t b = r % BN;
        r /= BN;
        const int64_t kl = r % G;
        r /= G;
        const int64_t ky = (r % ngroups) * G + kl, kz = r / ngroups;
        const float *k = ks ? ks[inst] : k1;
        const float *krow = ky < A1.K ? k + tap_source(kz, A0.K, reverse) * A0.ks + tap_source(ky, A1.K, reverse) * A1.ks
                                      : nullptr;
        for (int64_t c = lane; c < Cp; c += 32) {
            float w = 0.f;
            const int64_t off = c - b * A2.s;
            if (krow && off >= 0 && off % A2.d == 0 && off / A2.d < A2.K) {
                w = krow[tap_source(off / A2.d, A2.K, reverse) * A2.ks];
                if (!isfinite(w)) bad = true;
            }
            const __nv_bfloat16 h = __float2bfloat16_rn(w);
            hi[row * Cp + c] = h;
            lo[row * Cp + c] = __float2bfloat16_rn(w - __bfloat162float(h));
        }
    }
    return bad;
}

// Both pre-passes in one launch: blocks [0, nbs) split the data, the rest
// write the Toeplitz bands.  Every block stores whether it saw a non-finite
// value in flags[blockIdx.x] (no zeroing needed before the launch).
__global__ void __launch_bounds__(256) prepass_kernel(const float *__restrict__ x, const float *const *xs,
                                                      const float *__restrict__ k1, const float *const *ks,
                                                      int64_t n, Geom3<float> g, int64_t W, int64_t rows,
                                                      int64_t hop, int64_t lim, int reverse, int G,
                                                      int BN, int ngroups, int64_t Cp, __nv_bfloat16 *xh,
                                                      __nv_bfloat16 *xl, __nv_bfloat16 *th, __nv_bfloat16 *tl,
                                                      int nbs, int *flags) {
    const int b = blockIdx.x;
    const bool bad = b < nbs ? split_part(x, xs, n, g, W, rows, hop, lim, xh, xl, b, nbs)
                             : toeplitz_part(k1, ks, n, g, reverse, G, BN, ngroups, Cp, th, tl, b - nbs,
                                             (int64_t)gridDim.x - nbs);
    const int any = __syncthreads_or(bad);
    if (threadIdx.x == 0) flags[b] = any;
    // the flag array is read as 16-byte vectors: block 0 zeroes its padding
    if (b == 0 && threadIdx.x > 0 && threadIdx.x < 4 && (int)gridDim.x + (int)threadIdx.x - 1 < ((gridDim.x + 3) & ~3u))
        flags[gridDim.x + threadIdx.x - 1] = 0;
}

// ---- main kernel ----------------------------------------------------------
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
// Named barriers of the epilogue warps: 1 (vote) and 2 over both groups
// (256 threads), 3 over group 0 (128 threads).
__device__ __forceinline__ bool epi_vote(bool pred) {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n barrier.cta.red.or.pred q, 1, 256, p;\n selp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)pred)
        : "memory");
    return r != 0;
}
__device__ __forceinline__ void epi_sync() { asm volatile("barrier.cta.sync 2, 256;" ::: "memory"); }
__device__ __forceinline__ void grp0_sync() { asm volatile("barrier.cta.sync 3, 128;" ::: "memory"); }

struct TileCoord {
    int64_t inst, oz, oy0, ox0;
};
// (32-bit division: the host keeps the tile count below 2^31)
template <int BN> __device__ __forceinline__ TileCoord tile_of(const Params &P, int64_t t) {
    const uint32_t ti = (uint32_t)P.tiles_inst;
    const uint32_t inst = (uint32_t)t / ti;
    const uint32_t tt = (uint32_t)t - inst * ti, nct = (uint32_t)P.nct, nrt = (uint32_t)P.nrt;
    const uint32_t r = tt / nct;
    TileCoord c;
    c.inst = inst;
    c.ox0 = (int64_t)(tt - r * nct) * BN;
    c.oy0 = (int64_t)(r % nrt) * P.mvalid;
    c.oz = r / nrt;
    return c;
}
__device__ __forceinline__ float *out_of(const Params &P, int64_t inst) { return P.ys ? P.ys[inst] : P.y; }

// Persistent and warp-specialised: CTA b takes tiles b, b + grid, ...; per
// tile the kernel-row groups are work items.  Warp 8 (one lane) streams the
// items' stages through the TMA ring, warp 9 (one lane) issues the MMAs of
// item j into TMEM buffer j % 2, warps 0-7 drain buffer j % 2 (the shifted
// sums: warp shuffles, or a row block in shared memory; none with one kernel
// row per group at unit middle stride) while the MMAs of item j + 1 run in
// the other buffer.
template <int BN>
__global__ void __launch_bounds__(kThreads, 1)
    conv_kernel(const __grid_constant__ CUtensorMap tX_hi, const __grid_constant__ CUtensorMap tX_lo,
                const __grid_constant__ CUtensorMap tT_hi, const __grid_constant__ CUtensorMap tT_lo,
                const __grid_constant__ Params P) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    float *R = reinterpret_cast<float *>(base + P.ring_bytes);  // [2][BM][RP]
    uint64_t *full = reinterpret_cast<uint64_t *>(base + P.ring_bytes + kRowBlockBytes);
    uint64_t *empty = full + kMaxStages;
    uint64_t *tfull = empty + kMaxStages;
    uint64_t *tempty = tfull + 2;
    uint64_t *mdone = tempty + 2;
    uint64_t *bfull = mdone + 1;  // resident Toeplitz tiles loaded
    uint64_t *bfree = bfull + 1;  // resident Toeplitz tiles no longer read
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bfree + 1);
    int *bad = reinterpret_cast<int *>(tmem_slot + 1);     // some wait ran out
    int *issued_out = bad + 1;                              // the producer's stage count
    int *b_issued = issued_out + 1;                         // the producer's resident loads
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // CTA b takes the contiguous tiles [t0, t1) (tiles are instance-major, so
    // a CTA meets few instances and reloads resident Toeplitz tiles rarely)
    const int64_t per_cta = (P.ntiles + gridDim.x - 1) / gridDim.x;
    const int64_t t0 = (int64_t)blockIdx.x * per_cta, t1 = min(P.ntiles, t0 + per_cta);

    int nonfinite = 0;
    for (int i = tid; 4 * i < P.nflags; i += kThreads) {
        const int4 f = reinterpret_cast<const int4 *>(P.flags)[i];
        nonfinite |= f.x | f.y | f.z | f.w;
    }
    if (__syncthreads_or(nonfinite)) {
        // non-finite input somewhere: the FP32 direct loop for this CTA's tiles
        for (int64_t t = t0; t < t1; t++) {
            const TileCoord c = tile_of<BN>(P, t);
            const float *x = P.xs ? P.xs[c.inst] : P.x, *k = P.ks ? P.ks[c.inst] : P.k;
            float *y = out_of(P, c.inst);
            for (int u = tid; u < P.mvalid * BN; u += kThreads) {
                const int64_t oy = c.oy0 + u / BN, ox = c.ox0 + u % BN;
                if (oy < P.out1 && ox < (oy == P.out1 - 1 ? P.xlast : P.out2))
                    direct_naive_one<float>(x, k, y, P.dp, (c.oz * P.out1 + oy) * P.out2 + ox);
            }
        }
        return;
    }

    if (tid == 0) {
        for (int s = 0; s < P.stages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], 8);  // one arrival per epilogue warp
        }
        mbar_init(mdone, 1);
        mbar_init(bfull, 1);
        mbar_init(bfree, 1);
        *bad = 0;
        *issued_out = 0;
        *b_issued = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 9) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(2 * P.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    volatile int *vbad = bad;
    const int per_group = P.K0 * P.nchunk;

    if (warp == 8) {
        if (lane == 0) {
            // producer: data boxes (shared by a group's kernel rows) and the
            // Toeplitz tiles -- in each stage, or kept resident per instance
            // (every row group's) when they fit beside two data stages
            const int b_bytes = P.N * KC * 2;
            int it = 0, bl = 0;
            int64_t cur = -1;  // instance whose Toeplitz tiles are resident
            bool ok = true;
            for (int64_t t = t0; t < t1 && ok && !*vbad; t++) {
                const TileCoord c = tile_of<BN>(P, t);
                const int xb = (int)(c.ox0 * P.s2);
                if (P.bres && c.inst != cur) {
                    // (re)load the instance's tiles once the MMAs reading the
                    // previous instance's have finished
                    if (bl > 0 && !mbar_wait(bfree, (bl - 1) & 1)) {
                        atomicOr(bad, 1);
                        break;
                    }
                    mbar_expect_tx(bfull, P.ngroups * per_group * 2 * b_bytes);
                    for (int g = 0; g < P.ngroups; g++)
                        for (int i = 0; i < per_group; i++) {
                            const int kz = i / P.nchunk, ch = i % P.nchunk;
                            unsigned char *bs = base + P.b_off + (g * per_group + i) * 2 * b_bytes;
                            const int trow = (int)(c.inst * P.Rt) + (kz * P.ngroups + g) * P.N;
                            tma_2d(bs, &tT_hi, ch * KC, trow, bfull);
                            tma_2d(bs + b_bytes, &tT_lo, ch * KC, trow, bfull);
                        }
                    cur = c.inst;
                    *b_issued = ++bl;
                }
                for (int g = 0; g < P.ngroups && ok; g++) {
                    const int rb = (int)(c.oy0 * P.s1 + (int64_t)g * P.G * P.d1);
                    for (int i = 0; i < per_group; i++, it++) {
                        const int s = it % P.stages;
                        if (it >= P.stages && !mbar_wait(&empty[s], ((it / P.stages) - 1) & 1)) {
                            atomicOr(bad, 1);
                            ok = false;
                            break;
                        }
                        const int kz = i / P.nchunk, ch = i % P.nchunk;
                        unsigned char *st = base + s * P.stage_bytes;
                        mbar_expect_tx(&full[s], P.stage_bytes);
                        const int z = (int)(c.inst * P.P0 + c.oz * P.s0 + (int64_t)kz * P.d0);
                        tma_3d(st, &tX_hi, xb + ch * KC, rb, z, &full[s]);
                        tma_3d(st + A_BYTES, &tX_lo, xb + ch * KC, rb, z, &full[s]);
                        if (!P.bres) {
                            const int trow = (int)(c.inst * P.Rt) + (kz * P.ngroups + g) * P.N;
                            tma_2d(st + 2 * A_BYTES, &tT_hi, ch * KC, trow, &full[s]);
                            tma_2d(st + 2 * A_BYTES + b_bytes, &tT_lo, ch * KC, trow, &full[s]);
                        }
                    }
                }
            }
            *issued_out = it;
        }
    } else if (warp == 9) {
        if (lane == 0) {
            // MMA issuer: three split products per 16-wide K step, item j into buffer j % 2
            const int b_bytes = P.N * KC * 2;
            int it = 0, j = 0, bl = 0;
            int64_t cur = -1;
            bool ok = true;
            for (int64_t t = t0; t < t1 && ok && !*vbad; t++) {
                if (P.bres) {
                    const int64_t inst = (uint32_t)t / (uint32_t)P.tiles_inst;
                    if (inst != cur) {
                        // the previous instance's tiles are free once its MMAs finish
                        if (bl > 0) mma_commit(bfree);
                        if (!mbar_wait(bfull, bl & 1)) {
                            atomicOr(bad, 1);
                            break;
                        }
                        cur = inst;
                        bl++;
                    }
                }
                for (int g = 0; g < P.ngroups && ok; g++, j++) {
                    const int buf = j & 1;
                    if (j >= 2 && !mbar_wait(&tempty[buf], ((j >> 1) - 1) & 1)) {
                        atomicOr(bad, 1);
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t d = tmem + (uint32_t)(buf * P.tmem_cols);
                    for (int i = 0; i < per_group; i++, it++) {
                        const int s = it % P.stages;
                        if (!mbar_wait(&full[s], (it / P.stages) & 1)) {
                            atomicOr(bad, 1);
                            ok = false;
                            break;
                        }
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        const uint32_t sa = smem_u32(base + s * P.stage_bytes);
                        const uint32_t a_hi = sa, a_lo = sa + A_BYTES;
                        const uint32_t b_hi =
                            P.bres ? smem_u32(base + P.b_off + (g * per_group + i) * 2 * b_bytes) : sa + 2 * A_BYTES;
                        const uint32_t b_lo = b_hi + b_bytes;
                        const int nk = (i % P.nchunk == P.nchunk - 1) ? P.klast : KC / 16;
                        // a K step of 16 bf16 moves 32 bytes along the swizzled
                        // rows: 2 in the descriptors' start-address field
                        const uint64_t dah = sw128_desc(a_hi), dal = sw128_desc(a_lo);
                        const uint64_t dbh = sw128_desc(b_hi), dbl = sw128_desc(b_lo);
                        auto kstep = [&](int kk) {
                            const uint64_t o = (uint64_t)(2 * kk);
                            mma_bf16(d, dah + o, dbh + o, P.idesc, (i | kk) != 0);
                            mma_bf16(d, dah + o, dbl + o, P.idesc, 1);
                            mma_bf16(d, dal + o, dbh + o, P.idesc, 1);
                        };
                        if (nk == KC / 16) {
#pragma unroll
                            for (int kk = 0; kk < KC / 16; kk++) kstep(kk);
                        } else {
                            for (int kk = 0; kk < nk; kk++) kstep(kk);
                        }
                        mma_commit(&empty[s]);  // stage reusable once these MMAs have read it
                    }
                    if (!ok) break;
                    mma_commit(&tfull[buf]);  // buffer ready once the item's MMAs finish
                }
            }
            // every MMA issued has finished before the CTA moves on
            mma_commit(mdone);
            if (!mbar_wait(mdone, 0)) atomicOr(bad, 1);
        }
    } else {
        // epilogue: two groups of four warps (eg = warp / 4); warp w reads
        // TMEM lanes 32 (w % 4) .. +31 (tile rows).  Output row y of the tile
        // sums the kernel rows kl of the item at rows y s1 + kl d1; group eg
        // takes the rows kl = eg, eg + 2, ... and group 0 combines and
        // stores.  With one kernel row per group at unit middle stride
        // (row_epi) there is nothing to combine: group eg sums and stores
        // the 16-column blocks eg, eg + 2, ... of its rows.
        const int eg = warp >> 2, et = tid & 127, ew = warp & 3;
        const uint32_t lane_base = (uint32_t)(ew * 32) << 16;
        float *X0 = R, *X1 = R + BM * RP, *X2 = R + 2 * BM * RP;  // exchange blocks
        float acc[BN];
        int j = 0, rbuf = 0;
        bool stop = false;
        for (int64_t t = t0; t < t1 && !stop; t++) {
            const TileCoord c = tile_of<BN>(P, t);
#pragma unroll
            for (int q = 0; q < BN; q++) acc[q] = 0.f;
            for (int g = 0; g < P.ngroups; g++, j++) {
                const int buf = j & 1;
                const bool late = !mbar_wait(&tfull[buf], (j >> 1) & 1);
                if (epi_vote(late || *vbad)) {
                    if (late) atomicOr(bad, 1);
                    stop = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t tb = tmem + lane_base + (uint32_t)(buf * P.tmem_cols);
                if (P.row_epi) {
                    // no shifted sum: each group takes alternate 16-column
                    // blocks of its lanes' rows (no exchange, no barrier)
#pragma unroll
                    for (int bc = 0; bc < BN / 16; bc++) {
                        if ((bc & 1) != eg) continue;
                        float v[16];
                        tmem_ld16(tb + (uint32_t)(bc * 16), v);
#pragma unroll
                        for (int q = 0; q < 16; q++) acc[bc * 16 + q] += v[q];
                    }
                } else if (P.shfl_epi) {
                    // unit middle stride, row shifts kl d1 < 32: lane l takes the
                    // value of lane (l + kl d1) mod 32 of its own warp -- its own
                    // output's term when l + kl d1 < 32, else a term of output
                    // row l of the warp below (kept in spill); the partial sums
                    // meet in shared memory once per 16 columns
#pragma unroll
                    for (int bc = 0; bc < BN / 16; bc++) {
                        float own[16], spill[16];
#pragma unroll
                        for (int q = 0; q < 16; q++) own[q] = spill[q] = 0.f;
                        auto sum_row = [&](const uint32_t *v, int kl) {
                            const int sh = (int)(kl * P.d1);
                            if (sh == 0) {
#pragma unroll
                                for (int q = 0; q < 16; q++) own[q] += __uint_as_float(v[q]);
                                return;
                            }
                            const int src = (lane + sh) & 31;
                            const bool mine = lane + sh < 32;
#pragma unroll
                            for (int q = 0; q < 16; q++) {
                                const float a = __shfl_sync(0xffffffffu, __uint_as_float(v[q]), src);
                                if (mine) own[q] += a;
                                else spill[q] += a;
                            }
                        };
                        // the next row's TMEM load is in flight while a row is summed
                        uint32_t va[16], vb[16];
                        int kl = eg;
                        if (kl < P.G) {
                            tmem_ld16_issue(tb + (uint32_t)(kl * BN + bc * 16), va);
                            tmem_ld_wait(va);
                        }
                        for (; kl < P.G; kl += 4) {
                            const bool more = kl + 2 < P.G;
                            if (more) tmem_ld16_issue(tb + (uint32_t)((kl + 2) * BN + bc * 16), vb);
                            sum_row(va, kl);
                            if (more) {
                                tmem_ld_wait(vb);
                                const bool more2 = kl + 4 < P.G;
                                if (more2) tmem_ld16_issue(tb + (uint32_t)((kl + 4) * BN + bc * 16), va);
                                sum_row(vb, kl + 2);
                                if (more2) tmem_ld_wait(va);
                            }
                        }
                        // group 1: own -> X0, spill -> X1; group 0: spill -> X2
                        float4 *d0 = reinterpret_cast<float4 *>((eg ? X1 : X2) + et * RP);
#pragma unroll
                        for (int q = 0; q < 4; q++)
                            d0[q] = make_float4(spill[4 * q], spill[4 * q + 1], spill[4 * q + 2], spill[4 * q + 3]);
                        if (eg) {
                            float4 *d1 = reinterpret_cast<float4 *>(X0 + et * RP);
#pragma unroll
                            for (int q = 0; q < 4; q++)
                                d1[q] = make_float4(own[4 * q], own[4 * q + 1], own[4 * q + 2], own[4 * q + 3]);
                        }
                        epi_sync();
                        if (!eg) {
                            auto add = [&](const float *blk, int row) {
                                const float4 *s4 = reinterpret_cast<const float4 *>(blk + row * RP);
#pragma unroll
                                for (int q = 0; q < 4; q++) {
                                    const float4 u = s4[q];
                                    own[4 * q] += u.x;
                                    own[4 * q + 1] += u.y;
                                    own[4 * q + 2] += u.z;
                                    own[4 * q + 3] += u.w;
                                }
                            };
                            add(X0, et);
                            if (ew < 3) {
                                add(X2, et + 32);
                                add(X1, et + 32);
                            }
#pragma unroll
                            for (int q = 0; q < 16; q++) acc[bc * 16 + q] += own[q];
                        }
                        epi_sync();  // the blocks are rewritten for the next 16 columns
                    }
                } else if (!eg) {
                    // any stride: the rows pass through a double-buffered row
                    // block, one kernel row at a time (group 0 alone)
#pragma unroll
                    for (int bc = 0; bc < BN / 16; bc++) {
                        for (int kl = 0; kl < P.G; kl++, rbuf ^= 1) {
                            float v[16];
                            tmem_ld16(tb + (uint32_t)(kl * BN + bc * 16), v);
                            float *Rb = R + rbuf * (BM * RP);
                            float4 *dst = reinterpret_cast<float4 *>(Rb + et * RP);
#pragma unroll
                            for (int q = 0; q < 4; q++)
                                dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                            grp0_sync();
                            if (et < P.mvalid) {
                                const int r = (int)(et * P.s1 + kl * P.d1);  // < BM by the choice of mvalid
                                const float4 *src = reinterpret_cast<const float4 *>(Rb + r * RP);
#pragma unroll
                                for (int q = 0; q < 4; q++) {
                                    const float4 u = src[q];
                                    acc[bc * 16 + 4 * q] += u.x;
                                    acc[bc * 16 + 4 * q + 1] += u.y;
                                    acc[bc * 16 + 4 * q + 2] += u.z;
                                    acc[bc * 16 + 4 * q + 3] += u.w;
                                }
                            }
                        }
                    }
                }
                // buffer free for item j + 2
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&tempty[buf]);
            }
            if (!stop && (!eg || P.row_epi) && et < P.mvalid && c.oy0 + et < P.out1) {
                const int64_t xl = c.oy0 + et == P.out1 - 1 ? P.xlast : P.out2;  // columns of this row
                float *yr = out_of(P, c.inst) + c.oz * P.ys0 + (c.oy0 + et) * P.ys1 + c.ox0;
                if (P.row_epi) {
                    // each group stores the 16-column blocks it summed
#pragma unroll
                    for (int bc = 0; bc < BN / 16; bc++) {
                        if ((bc & 1) != eg) continue;
                        float *yb = yr + bc * 16;
                        if (c.ox0 + bc * 16 + 16 <= xl && (reinterpret_cast<uintptr_t>(yb) & 15) == 0) {
#pragma unroll
                            for (int q = 0; q < 4; q++)
                                reinterpret_cast<float4 *>(yb)[q] =
                                    make_float4(acc[bc * 16 + 4 * q], acc[bc * 16 + 4 * q + 1],
                                                acc[bc * 16 + 4 * q + 2], acc[bc * 16 + 4 * q + 3]);
                        } else {
#pragma unroll
                            for (int q = 0; q < 16; q++)
                                if (c.ox0 + bc * 16 + q < xl) yb[q] = acc[bc * 16 + q];
                        }
                    }
                } else if (c.ox0 + BN <= xl && (reinterpret_cast<uintptr_t>(yr) & 15) == 0) {
#pragma unroll
                    for (int q = 0; q < BN / 4; q++)
                        reinterpret_cast<float4 *>(yr)[q] =
                            make_float4(acc[4 * q], acc[4 * q + 1], acc[4 * q + 2], acc[4 * q + 3]);
                } else {
#pragma unroll
                    for (int q = 0; q < BN; q++)
                        if (c.ox0 + q < xl) yr[q] = acc[q];
                }
            }
        }
    }
    __syncwarp();  // the producer and MMA warps reconverge after their single-lane roles
    __syncthreads();
    if (*vbad) {
        // a pipeline wait ran out (not expected): this CTA's tiles become NaN
        // and the per-device word keeps the event.  Before the shared memory
        // and TMEM are released, the loads already issued must have landed
        // (the MMAs issued have finished: mdone); waits bounded as well.
        if (tid == 0) {
            const int issued = *issued_out;
            for (int i = issued > P.stages ? issued - P.stages : 0; i < issued; i++)
                mbar_wait(&full[i % P.stages], (i / P.stages) & 1);
            if (*b_issued > 0) mbar_wait(bfull, (*b_issued - 1) & 1);
            atomicOr(&g_timeouts, 1);
        }
        for (int64_t t = t0; t < t1; t++) {
            const TileCoord c = tile_of<BN>(P, t);
            float *y = out_of(P, c.inst);
            for (int u = tid; u < P.mvalid * BN; u += kThreads) {
                const int64_t oy = c.oy0 + u / BN, ox = c.ox0 + u % BN;
                if (oy < P.out1 && ox < (oy == P.out1 - 1 ? P.xlast : P.out2))
                    y[c.oz * P.ys0 + oy * P.ys1 + ox] = __int_as_float(0x7fc00000);
            }
        }
        __syncthreads();
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 9) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * P.tmem_cols)
                     : "memory");
    }
}

// ---- Complex<f32> as four real convolutions -------------------------------
// Device arrays of the four real instances' pointers (written by a kernel so
// that the call stays capturable into a CUDA graph).
__global__ void set_ptrs_kernel(const float **xs, const float **ks, float **ys, const float *x0, const float *x1,
                                const float *x2, const float *x3, const float *k0, const float *k1, const float *k2,
                                const float *k3, float *y0, float *y1, float *y2, float *y3) {
    xs[0] = x0; xs[1] = x1; xs[2] = x2; xs[3] = x3;
    ks[0] = k0; ks[1] = k1; ks[2] = k2; ks[3] = k3;
    ys[0] = y0; ys[1] = y1; ys[2] = y2; ys[3] = y3;
}

// y = (xr kr - xi ki) + i (xr ki + xi kr) from the four real results
__global__ void complex_combine_kernel(const float *__restrict__ rr, const float *__restrict__ ii,
                                       const float *__restrict__ ri, const float *__restrict__ ir,
                                       float2 *__restrict__ y, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = make_float2(rr[i] - ii[i], ri[i] + ir[i]);
}

// ---- host -------------------------------------------------------------------
typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
    static EncodeTiled fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    });
    return fn;
}

int make_map(CUtensorMap *m, void *base, int rank, const cuuint64_t *dims, const cuuint64_t *strides_b,
             const cuuint32_t *box) {
    EncodeTiled enc = encoder();
    if (!enc) return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, base, dims, strides_b, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "tensor map encoding failed");
    return NDCONV_OK;
}

// Tile plan of one problem.
struct TilePlan {
    int G, ngroups, BN, N;
    int64_t Kpad;  // K extent of one row correlation (multiple of 16)
    int nchunk, klast;
    int mvalid;
    int stages, stage_bytes, ring_bytes, smem;
    int bres, b_off;
};

inline int64_t kpad_of(const AxisGeom &A2, int BN) {
    return ((BN - 1) * A2.s + (A2.K - 1) * A2.d + 1 + 15) / 16 * 16;
}

// Kernel rows per group: at most 16, and few enough that (G - 1) d1 leaves
// at least half of the 128 staged rows as outputs; the groups are evened out.
// Output columns per tile BN (16, 32 or 64, with G BN <= 256): the
// autotuner's choice when it fits, else the one with the least modelled MMA
// time per output -- an MMA of N columns costs max(N / 2, (4096 + 32 N) / 128)
// cycles (tensor rate, or shared-memory reads of its two operands).
TilePlan plan_tiles(const Plan3 &P) {
    const AxisGeom *A = P.ax;
    TilePlan t{};
    int G = (int)std::min<int64_t>(A[1].K, 16);
    while (G > 1 && (G - 1) * A[1].d > 63) G--;
    t.ngroups = (int)((A[1].K + G - 1) / G);
    t.G = (int)((A[1].K + t.ngroups - 1) / t.ngroups);
    double best = 1e300;
    for (int bn = 16; bn <= 64; bn *= 2) {
        if (t.G * bn > 256) break;
        const int n = t.G * bn;
        const double mma = std::max(n / 2.0, (4096.0 + 32.0 * n) / 128.0);
        const double cost = (double)(kpad_of(A[2], bn) / 16) * mma / bn;
        if (cost < best) {
            best = cost;
            t.BN = bn;
        }
    }
    const int want = ndconv_tune(NDCONV_TUNE_BF16X3_BN);
    if ((want == 16 || want == 32 || want == 64) && t.G * want <= 256) t.BN = want;
    t.N = t.G * t.BN;
    t.Kpad = kpad_of(A[2], t.BN);
    t.nchunk = (int)((t.Kpad + KC - 1) / KC);
    t.klast = (int)((t.Kpad - (int64_t)(t.nchunk - 1) * KC) / 16);
    t.mvalid = (int)((BM - 1 - (int64_t)(t.G - 1) * A[1].d) / A[1].s + 1);
    // a kernel whose Toeplitz tiles (every row group, plane tap and K chunk)
    // fit beside a ring of at least two data stages keeps them in shared
    // memory (per instance); the ring then streams only the data boxes
    const int bslot = 2 * t.N * KC * 2;
    const int64_t bres_bytes = (int64_t)t.ngroups * A[0].K * t.nchunk * bslot;
    t.bres = bres_bytes + 2 * (2 * A_BYTES) <= kSmemLimit - kSmemExtra;
    t.stage_bytes = 2 * A_BYTES + (t.bres ? 0 : bslot);
    t.stages = std::min<int64_t>(kMaxStages, (kSmemLimit - kSmemExtra - (t.bres ? bres_bytes : 0)) / t.stage_bytes);
    t.b_off = t.stages * t.stage_bytes;
    t.ring_bytes = t.b_off + (t.bres ? (int)bres_bytes : 0);
    t.smem = t.ring_bytes + kSmemExtra;
    return t;
}

// Which problems the split path takes (f32; all index ranges within the TMA
// coordinate range).
bool applies(const Plan3 &P) {
    const AxisGeom *A = P.ax;
    if (P.dtype != NDCONV_F32) return false;
    for (int a = 0; a < 3; a++)
        if (A[a].L > (1 << 30) || A[a].out < 1 || A[a].s > (1 << 20) || A[a].d > (1 << 20)) return false;
    return A[0].K * (2 * A[1].K + 16) * 64 < (1 << 30) && A[2].K * A[2].d < (1 << 28) &&
           A[0].L * A[1].L < 0x7fffffff;
}

// A single row (a 1-D signal, or an array of one row with one-row kernels)
// folds into R virtual rows of S outputs: virtual row r starts at padded
// position r S s2, so the 128 accumulator lanes of a tile hold 128 stretches
// of the row instead of one row and 127 lanes of padding.  S is the least
// multiple of BN that is at least 4 (K2 - 1) d2 / s2: neighbouring stretches
// share (K2 - 1) d2 + 1 - s2 inputs, at most about a fifth of a virtual row.
struct RowFold {
    int64_t S = 0;      // outputs per virtual row (0: not folded)
    int64_t R = 1;      // virtual rows
    int64_t hop = 0;    // padded positions between virtual rows (S s2)
    int64_t xlast = 0;  // outputs in the last output row
};
Plan3 fold_row(const Plan3 &P, int BN, RowFold *f) {
    const AxisGeom *A = P.ax;
    *f = RowFold{};
    f->xlast = A[2].out;
    if (!(A[0].L == 1 && A[1].L == 1 && A[0].K == 1 && A[1].K == 1 && A[0].out == 1 && A[1].out == 1)) return P;
    const int64_t want = (4 * (A[2].K - 1) * A[2].d + A[2].s - 1) / A[2].s;
    const int64_t S = std::max<int64_t>(BN, (want + BN - 1) / BN * BN);
    const int64_t R = (A[2].out + S - 1) / S;
    if (R < 2) return P;  // one stretch: nothing to fold
    Plan3 V = P;
    AxisGeom &v1 = V.ax[1], &v2 = V.ax[2];
    v1.n = v1.L = v1.out = R;
    v1.p0 = v1.p1 = 0;
    v1.K = v1.d = v1.keff = v1.s = 1;
    v2.out = S;
    v2.L = v2.n = (S - 1) * A[2].s + (A[2].K - 1) * A[2].d + 1;
    v2.p0 = v2.p1 = 0;
    v2.keff = (A[2].K - 1) * A[2].d + 1;
    f->S = S;
    f->R = R;
    f->hop = S * A[2].s;
    f->xlast = A[2].out - (R - 1) * S;
    return V;
}

// The plan a call runs: the problem's own geometry, or its folded row.
Plan3 tile_geometry(const Plan3 &P, TilePlan *T, RowFold *f) {
    const Plan3 V = fold_row(P, plan_tiles(P).BN, f);
    *T = plan_tiles(V);
    return V;
}

}  // namespace bf16x3

bool bf16x3_applies(const Plan3 &P) { return bf16x3::applies(P); }

}  // namespace ndconv

using namespace ndconv;
using namespace ndconv::bf16x3;

namespace {
// n instances of one geometry: pointers x / k / y for one instance, or
// device arrays xs / ks / ys of n pointers each.  The padded planes and
// Toeplitz bands of all instances live in one workspace; one persistent
// launch covers every instance's tiles.
int run_bf16x3(const ndconv_problem *p, int64_t n, const float *x, const float *k, float *y,
               const float *const *xs, const float *const *ks, float *const *ys, cudaStream_t st) {
    Plan3 P;
    int s = plan_problem(p, 0, &P);
    if (s) return s;
    if (!applies(P)) return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "3xBF16 path: f32 within the TMA index range only");
    const Geom3<float> g = P.geom<float>();  // where the samples come from
    TilePlan T;
    RowFold f;
    const Plan3 V = tile_geometry(P, &T, &f);  // what the tiles cover
    const AxisGeom *A = V.ax;
    const int64_t Cp = (int64_t)T.nchunk * KC;                  // Toeplitz row pitch (elements)
    const int64_t W = std::max<int64_t>(KC, (A[2].L + 7) / 8 * 8);  // data row pitch (16-byte multiple)
    const int64_t Rt = A[0].K * T.ngroups * T.N;                // Toeplitz rows per instance
    const size_t nX = (size_t)(n * A[0].L * A[1].L * W), nT = (size_t)(n * Rt * Cp);
    const int64_t nrt = (A[1].out + T.mvalid - 1) / T.mvalid, nct = (A[2].out + T.BN - 1) / T.BN;
    const int64_t tiles_inst = A[0].out * nrt * nct, ntiles = n * tiles_inst;
    if (ntiles >= 0x7fffffff || n * A[0].L >= 0x7fffffff || n * Rt >= 0x7fffffff)
        return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "batch beyond the 32-bit tile and TMA coordinate range");
    int dev = 0, nsm = 0;
    NDCONV_CUDA_OK(cudaGetDevice(&dev));
    NDCONV_CUDA_OK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int64_t gx = std::min<int64_t>(ntiles, nsm);  // persistent: one CTA per SM
    unsigned char *ws = nullptr;
    // pre-pass blocks: data split, then Toeplitz rows (one warp each)
    const int64_t items = n * A[0].L * A[1].L * (W / 8), trows = n * Rt;
    const int nbs = (int)std::max<int64_t>(1, std::min<int64_t>(16 * nsm, (items + 255) / 256));
    const int nbt = (int)std::max<int64_t>(1, std::min<int64_t>(16 * nsm, (trows + 7) / 8));
    const int nflags = (nbs + nbt + 3) & ~3;  // padded to whole 16-byte vectors
    const size_t bytes = 2 * sizeof(__nv_bfloat16) * (nX + nT) + sizeof(int) * (size_t)nflags + 256;
    cudaError_t e = cudaMallocAsync((void **)&ws, bytes, st);
    if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_NO_MEMORY, cudaGetErrorString(e));
    __nv_bfloat16 *xh = reinterpret_cast<__nv_bfloat16 *>(ws), *xl = xh + nX, *th = xl + nX, *tl = th + nT;
    int *flags = reinterpret_cast<int *>(tl + nT);
    flags = reinterpret_cast<int *>((reinterpret_cast<uintptr_t>(flags) + 15) & ~(uintptr_t)15);
    auto fail = [&](int code) {
        cudaFreeAsync(ws, st);
        return code;
    };
    CUtensorMap mXh, mXl, mTh, mTl;
    {
        const cuuint64_t dX[3] = {(cuuint64_t)W, (cuuint64_t)A[1].L, (cuuint64_t)(n * A[0].L)};
        const cuuint64_t sX[2] = {(cuuint64_t)W * 2, (cuuint64_t)(W * A[1].L * 2)};
        const cuuint32_t bX[3] = {KC, BM, 1};
        const cuuint64_t dT[2] = {(cuuint64_t)Cp, (cuuint64_t)(n * Rt)};
        const cuuint64_t sT[1] = {(cuuint64_t)Cp * 2};
        const cuuint32_t bT[2] = {KC, (cuuint32_t)T.N};
        if ((s = make_map(&mXh, xh, 3, dX, sX, bX)) || (s = make_map(&mXl, xl, 3, dX, sX, bX)) ||
            (s = make_map(&mTh, th, 2, dT, sT, bT)) || (s = make_map(&mTl, tl, 2, dT, sT, bT)))
            return fail(s);
    }
    prepass_kernel<<<nbs + nbt, 256, 0, st>>>(x, xs, k, ks, n, g, W, A[0].L * A[1].L, f.hop, A[2].L, P.reverse,
                                             T.G, T.BN, T.ngroups, Cp, xh, xl, th, tl, nbs, flags);
    ndconv_count_launch();
    Params Q{};
    Q.out0 = A[0].out;
    Q.out1 = A[1].out;
    Q.out2 = A[2].out;
    Q.s0 = A[0].s;
    Q.d0 = A[0].d;
    Q.s1 = A[1].s;
    Q.d1 = A[1].d;
    Q.s2 = A[2].s;
    Q.K0 = (int)A[0].K;
    Q.G = T.G;
    Q.ngroups = T.ngroups;
    Q.N = T.N;
    Q.mvalid = T.mvalid;
    Q.nrt = nrt;
    Q.nct = nct;
    Q.ntiles = ntiles;
    Q.nchunk = T.nchunk;
    Q.klast = T.klast;
    Q.stages = T.stages;
    Q.stage_bytes = T.stage_bytes;
    Q.ring_bytes = T.ring_bytes;
    Q.bres = T.bres;
    Q.b_off = T.b_off;
    Q.row_epi = (T.G == 1 && A[1].s == 1) ? 1 : 0;
    Q.shfl_epi = (!Q.row_epi && A[1].s == 1 && (T.G - 1) * A[1].d < 32) ? 1 : 0;
    Q.tmem_cols = T.N <= 32 ? 32 : T.N <= 64 ? 64 : T.N <= 128 ? 128 : 256;
    Q.idesc = idesc_bf16(BM, T.N);
    Q.y = y;
    Q.ys0 = A[1].out * A[2].out;
    Q.ys1 = A[2].out;
    Q.xlast = f.xlast;
    Q.flags = flags;
    Q.nflags = nflags;
    Q.dp = P.direct<float>();
    Q.x = x;
    Q.k = k;
    Q.xs = xs;
    Q.ks = ks;
    Q.ys = ys;
    Q.tiles_inst = tiles_inst;
    Q.P0 = A[0].L;
    Q.Rt = Rt;
    const void *fn = T.BN == 16   ? (const void *)conv_kernel<16>
                     : T.BN == 32 ? (const void *)conv_kernel<32>
                                  : (const void *)conv_kernel<64>;
    e = ndconv_allow_smem(fn, T.smem);
    if (e != cudaSuccess) return fail(ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e)));
    const dim3 grid((unsigned)gx);
    if (T.BN == 16) conv_kernel<16><<<grid, kThreads, T.smem, st>>>(mXh, mXl, mTh, mTl, Q);
    else if (T.BN == 32) conv_kernel<32><<<grid, kThreads, T.smem, st>>>(mXh, mXl, mTh, mTl, Q);
    else conv_kernel<64><<<grid, kThreads, T.smem, st>>>(mXh, mXl, mTh, mTl, Q);
    ndconv_count_launch();
    e = cudaGetLastError();
    cudaFreeAsync(ws, st);  // stream-ordered: after the launch has finished with it
    if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
    return NDCONV_OK;
}
// Complex<f32>: the real and imaginary parts are strided f32 views of the
// interleaved arrays (element strides doubled, the imaginary part one float
// further); the padded real view takes the real part of each border
// constant, the imaginary view the imaginary part (the other border kinds
// commute with taking parts).  Batched launches give xr*kr, xr*ki (real view
// of the data) and xi*ki, xi*kr -- one launch when both views pad alike, two
// otherwise; a last pass combines them as num-complex's product does.
int run_bf16x3_complex(const ndconv_problem *p, const c32 *x, const c32 *k, c32 *y, cudaStream_t st) {
    Plan3 P;
    int s = plan_problem(p, 0, &P);
    if (s) return s;
    ndconv_problem q = *p;
    q.dtype = NDCONV_F32;
    const int r = p->rank;
    auto doubled = [&](const int64_t *shape, const int64_t *strides, int64_t *outs) {
        bool contig = true;
        for (int i = 0; i < r; i++) contig = contig && strides[i] == 0;
        int64_t run = 1;
        for (int i = r - 1; i >= 0; i--) {
            outs[i] = 2 * (contig ? run : strides[i]);
            run *= shape[i];
        }
    };
    doubled(p->data_shape, p->data_strides, q.data_strides);
    doubled(p->kernel_shape, p->kernel_strides, q.kernel_strides);
    ndconv_problem qi = q;  // the imaginary view: the constants' imaginary parts
    qi.const_value[0] = p->const_value[1];
    qi.const_value[1] = 0;
    q.const_value[1] = 0;
    for (int a = 0; a < 3; a++)
        for (int sd = 0; sd < 2; sd++) {
            qi.border_value[a][sd][0] = p->border_value[a][sd][1];
            qi.border_value[a][sd][1] = 0;
            q.border_value[a][sd][1] = 0;
        }
    Plan3 Q;
    if ((s = plan_problem(&q, 0, &Q))) return s;
    if (!applies(Q)) return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "3xBF16 path: beyond the TMA index range");
    const int64_t ny = P.ax[0].out * P.ax[1].out * P.ax[2].out;
    unsigned char *ws = nullptr;
    const size_t bytes = sizeof(float) * 4 * (size_t)ny + 3 * 4 * sizeof(void *) + 256;
    cudaError_t e = cudaMallocAsync((void **)&ws, bytes, st);
    if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_NO_MEMORY, cudaGetErrorString(e));
    float *t = reinterpret_cast<float *>(ws);  // rr, ri, ii, ir
    const float **xs = reinterpret_cast<const float **>(
        (reinterpret_cast<uintptr_t>(t + 4 * ny) + 15) & ~(uintptr_t)15);
    const float **ks = xs + 4;
    float **ys = reinterpret_cast<float **>(reinterpret_cast<uintptr_t>(ks + 4));
    const float *xr = reinterpret_cast<const float *>(x), *kr = reinterpret_cast<const float *>(k);
    set_ptrs_kernel<<<1, 1, 0, st>>>(xs, ks, ys, xr, xr, xr + 1, xr + 1, kr, kr + 1, kr + 1, kr, t, t + ny,
                                     t + 2 * ny, t + 3 * ny);
    ndconv_count_launch();
    // one launch for all four when both views pad alike (no constant has an
    // imaginary part that differs from its real part)
    bool alike = q.const_value[0] == qi.const_value[0];
    for (int a = 0; a < 3; a++)
        for (int sd = 0; sd < 2; sd++) alike = alike && q.border_value[a][sd][0] == qi.border_value[a][sd][0];
    if (alike) {
        s = run_bf16x3(&q, 4, nullptr, nullptr, nullptr, xs, ks, ys, st);
    } else {
        s = run_bf16x3(&q, 2, nullptr, nullptr, nullptr, xs, ks, ys, st);
        if (!s) s = run_bf16x3(&qi, 2, nullptr, nullptr, nullptr, xs + 2, ks + 2, ys + 2, st);
    }
    if (!s) {
        const unsigned nb = (unsigned)std::max<int64_t>(1, std::min<int64_t>(152 * 8, (ny + 255) / 256));
        complex_combine_kernel<<<nb, 256, 0, st>>>(t, t + 2 * ny, t + ny, t + 3 * ny, reinterpret_cast<float2 *>(y),
                                                   ny);
        ndconv_count_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) s = ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaFreeAsync(ws, st);
    return s;
}
}  // namespace

extern "C" int ndconv_conv_bf16x3(const ndconv_problem *p, const void *data, const void *kernel, void *out,
                                  void *stream) {
    if (!data || !kernel || !out) {
        Plan3 P;
        if (const int s = plan_problem(p, 0, &P)) return s;
        return ndconv_fail(NDCONV_ERR_INVALID, "null pointer");
    }
    if (p && p->dtype == NDCONV_C32)
        return run_bf16x3_complex(p, static_cast<const c32 *>(data), static_cast<const c32 *>(kernel),
                                  static_cast<c32 *>(out), (cudaStream_t)stream);
    return run_bf16x3(p, 1, static_cast<const float *>(data), static_cast<const float *>(kernel),
                      static_cast<float *>(out), nullptr, nullptr, nullptr, (cudaStream_t)stream);
}

// See include/ndconv.h.
extern "C" int ndconv_conv_bf16x3_batch(const ndconv_problem *p, int64_t n, const void *const *data,
                                        const void *const *kernel, void *const *out, void *stream) {
    Plan3 P;
    if (const int s = plan_problem(p, 0, &P)) return s;
    if (n < 0) return ndconv_fail(NDCONV_ERR_INVALID, "negative batch size");
    if (n == 0) return NDCONV_OK;
    if (!data || !kernel || !out) return ndconv_fail(NDCONV_ERR_INVALID, "null pointer array");
    return run_bf16x3(p, n, nullptr, nullptr, nullptr, reinterpret_cast<const float *const *>(data),
                      reinterpret_cast<const float *const *>(kernel), reinterpret_cast<float *const *>(out),
                      (cudaStream_t)stream);
}

// See include/ndconv.h.  Host only: the tile plan ndconv_conv_bf16x3 would
// launch for p (f32 geometry; a complex problem's plan is its real views').
extern "C" int ndconv_bf16x3_plan(const ndconv_problem *p, int64_t out[18]) {
    if (!out) return ndconv_fail(NDCONV_ERR_INVALID, "null output");
    ndconv_problem q = *p;
    if (q.dtype == NDCONV_C32) q.dtype = NDCONV_F32;
    Plan3 P;
    if (const int s = plan_problem(&q, 0, &P)) return s;
    if (!applies(P)) return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "3xBF16 path: f32 within the TMA index range only");
    TilePlan T;
    RowFold f;
    const Plan3 V = tile_geometry(P, &T, &f);
    const AxisGeom *A = V.ax;
    const int64_t v[18] = {T.G, T.ngroups, T.BN, T.N, T.Kpad, T.nchunk, T.klast, T.mvalid,
                           T.stages, T.stage_bytes, T.ring_bytes, T.smem, T.bres, (A[1].out + T.mvalid - 1) / T.mvalid,
                           (A[2].out + T.BN - 1) / T.BN, kSmemLimit, f.S, f.R};
    for (int i = 0; i < 18; i++) out[i] = v[i];
    return NDCONV_OK;
}

// See include/ndconv.h.  Waits for the stream, then reads and clears the
// device's timeout word.
extern "C" int ndconv_bf16x3_status(void *stream) {
    NDCONV_CUDA_OK(cudaStreamSynchronize((cudaStream_t)stream));
    int v = 0;
    const int zero = 0;
    NDCONV_CUDA_OK(cudaMemcpyFromSymbol(&v, ndconv::bf16x3::g_timeouts, sizeof(int)));
    if (v) NDCONV_CUDA_OK(cudaMemcpyToSymbol(ndconv::bf16x3::g_timeouts, &zero, sizeof(int)));
    if (v) return ndconv_fail(NDCONV_ERR_TIMEOUT, "a 3xBF16 tensor-core pipeline wait ran out (its tile holds NaN)");
    return NDCONV_OK;
}
