// Direct convolution on the 5th-generation tensor cores with 3xBF16 split
// products (f32 data and kernels, f32 accumulation in tensor memory).
//
// Each f32 value v is split as hi = bf16(v), lo = bf16(v - hi), and a
// product x k is formed as xh kh + xh kl + xl kh (the dropped xl kl term and
// the splits' rounding leave ~2^-16 relative error per product, below the
// 1e-5 normwise bar).  The convolution becomes one GEMM per output tile:
//   D[m][n] = sum over leading taps t = (kz, ky) and input offsets c of
//             T_t[m][c] * X_t[n][c]
// with m = 128 consecutive outputs along the contiguous axis (TMEM lanes),
// n = BN consecutive output rows (TMEM columns), T_t the Toeplitz band of
// kernel row t (T_t[m][c] = k[t][tx] when c = m s2 + tx d2), and X_t the
// padded data rows (oz s0 + kz d0, oy + ky d1) over the tile's input window.
// Both operands are K-major bf16 tiles of 64 elements (one 128-byte
// swizzled row) staged by TMA from two pre-built planes in global memory:
// the padded data (border map applied once, split into hi / lo) and the
// Toeplitz bands.  One thread issues TMA, one issues tcgen05.mma, all four
// warps drain TMEM with tcgen05.ld.  Every mbarrier wait is bounded; a
// timeout (not expected) writes NaN to the tile's outputs, records the event
// in a library-owned per-device word (read and cleared by
// ndconv_bf16x3_status), waits (bounded) for the tile's TMA loads and MMAs
// already in flight, and the CTA still releases TMEM.
// Non-finite inputs (bit 0, found by the pre-pass) make every CTA compute its
// tile with the FP32 direct loop instead, like the reference's sums.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "common.cuh"
#include "direct.h"
#include "direct_blocks.cuh"
#include "geometry.h"
#include "ndconv.h"

namespace ndconv {
namespace bf16x3 {

constexpr int BM = 128;  // outputs along the contiguous axis per tile (TMEM lanes)
constexpr int KC = 64;   // bf16 per K chunk: one 128-byte swizzled row
constexpr int A_BYTES = BM * KC * 2;
// BN output rows per tile (TMEM columns): 64, or 32 for problems whose
// 64-row tiles would leave SMs idle
template <int BN> struct Tile {
    static constexpr int B_BYTES = BN * KC * 2;
    static constexpr int STAGES = BN >= 64 ? 4 : 5;
    static constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
};
constexpr long long kWaitCycles = 2000000000LL;  // ~1 s of polling before a wait gives up
constexpr int kThreads = 128;

// Timeouts of any launch on this device since the last ndconv_bf16x3_status
// call (a file-scope device variable: one per device that loads the library).
__device__ int g_timeouts;

struct Params {
    int64_t out0, out1, out2;
    int64_t s0, d0, d1;
    int K0, K1;
    int nchunk;  // K chunks per leading tap
    int nseg;    // tiles along the contiguous axis
    int64_t s2;
    float *y;
    int64_t ys0, ys1;
    int *status;  // bit 0: non-finite input seen; bit 1: a wait ran out
    DirectParams<float> dp;  // FP32 fallback
    const float *x, *k;
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

// ---- pre-passes -----------------------------------------------------------
// Padded data planes [P0][P1][W] (hi, lo); zero beyond the padded extent.
__global__ void split_data_kernel(const float *__restrict__ x, Geom3<float> g, int64_t W,
                                  __nv_bfloat16 *__restrict__ hi, __nv_bfloat16 *__restrict__ lo, int *status) {
    const int64_t P1 = g.ax[1].L, P2 = g.ax[2].L;
    const int64_t total = g.ax[0].L * P1 * W;
    bool bad = false;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total;
         u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i2 = u % W, r = u / W;
        const int64_t i1 = r % P1, i0 = r / P1;
        float v = 0.f;
        if (i2 < P2)
            v = resolve_padded<float>(x, g, axis_map(g.ax[0], i0), axis_map(g.ax[1], i1), axis_map(g.ax[2], i2));
        if (!isfinite(v)) bad = true;
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        hi[u] = h;
        lo[u] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
    if (bad) atomicOr(status, 1);
}

// Toeplitz bands [K0 K1][BM][Cpad] (hi, lo): T_t[m][c] = kf[t][tx] where
// c = m s2 + tx d2 (kf: the kernel in tap order, reversed for convolution).
__global__ void toeplitz_kernel(const float *__restrict__ k, Geom3<float> g, int reverse, int64_t Cpad,
                                __nv_bfloat16 *__restrict__ hi, __nv_bfloat16 *__restrict__ lo, int *status) {
    const AxisGeom &A0 = g.ax[0], &A1 = g.ax[1], &A2 = g.ax[2];
    const int64_t total = A0.K * A1.K * BM * Cpad;
    bool bad = false;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total;
         u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = u % Cpad, r = u / Cpad;
        const int64_t m = r % BM, t = r / BM;
        const int64_t kz = t / A1.K, ky = t % A1.K;
        float w = 0.f;
        const int64_t off = c - m * A2.s;
        if (off >= 0 && off % A2.d == 0 && off / A2.d < A2.K) {
            const int64_t tx = off / A2.d;
            w = k[tap_source(kz, A0.K, reverse) * A0.ks + tap_source(ky, A1.K, reverse) * A1.ks +
                  tap_source(tx, A2.K, reverse) * A2.ks];
            if (!isfinite(w)) bad = true;
        }
        const __nv_bfloat16 h = __float2bfloat16_rn(w);
        hi[u] = h;
        lo[u] = __float2bfloat16_rn(w - __bfloat162float(h));
    }
    if (bad) atomicOr(status, 1);
}

// ---- main kernel ----------------------------------------------------------
template <int BN>
__global__ void __launch_bounds__(kThreads, 1)
    conv_kernel(const __grid_constant__ CUtensorMap tA_hi, const __grid_constant__ CUtensorMap tA_lo,
                const __grid_constant__ CUtensorMap tB_hi, const __grid_constant__ CUtensorMap tB_lo,
                const __grid_constant__ Params P) {
    constexpr int STAGES = Tile<BN>::STAGES, STAGE_BYTES = Tile<BN>::STAGE_BYTES, B_BYTES = Tile<BN>::B_BYTES;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(base + STAGES * STAGE_BYTES);
    uint64_t *empty = full + STAGES;
    uint64_t *done = empty + STAGES;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    int *bad = reinterpret_cast<int *>(tmem_slot + 1);  // a role's wait ran out
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int q = blockIdx.x % P.nseg;          // tile along the contiguous axis
    const int64_t oy0 = (int64_t)(blockIdx.x / P.nseg) * BN;
    const int64_t oz = blockIdx.y;

    if (*reinterpret_cast<volatile int *>(P.status) & 1) {
        // non-finite input somewhere: the FP32 direct loop for this tile
        for (int u = tid; u < BM * BN; u += kThreads) {
            const int64_t ox = (int64_t)q * BM + (u % BM), oy = oy0 + u / BM;
            if (ox < P.out2 && oy < P.out1)
                direct_naive_one<float>(P.x, P.k, P.y, P.dp, (oz * P.out1 + oy) * P.out2 + ox);
        }
        return;
    }

    if (tid == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *bad = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const int niter = P.K0 * P.K1 * P.nchunk;

    int issued = 0;  // producer: K steps whose TMA loads were issued
    if (tid == 0) {
        // producer: Toeplitz band tiles and data row tiles
        const int x0 = (int)((int64_t)q * BM * P.s2);
        for (int i = 0; i < niter; i++) {
            const int s = i % STAGES;
            if (i >= STAGES && !mbar_wait(&empty[s], ((i / STAGES) - 1) & 1)) {
                atomicOr(bad, 1);
                break;
            }
            const int t = i / P.nchunk, c = i % P.nchunk;
            const int kz = t / P.K1, ky = t % P.K1;
            unsigned char *st = base + s * STAGE_BYTES;
            mbar_expect_tx(&full[s], STAGE_BYTES);
            tma_2d(st, &tA_hi, c * KC, t * BM, &full[s]);
            tma_2d(st + A_BYTES, &tA_lo, c * KC, t * BM, &full[s]);
            const int by = (int)(oy0 + (int64_t)ky * P.d1), bz = (int)(oz * P.s0 + (int64_t)kz * P.d0);
            tma_3d(st + 2 * A_BYTES, &tB_hi, x0 + c * KC, by, bz, &full[s]);
            tma_3d(st + 2 * A_BYTES + B_BYTES, &tB_lo, x0 + c * KC, by, bz, &full[s]);
            issued = i + 1;
        }
    } else if (tid == 32) {
        // MMA issuer: three split products per 16-wide K step
        constexpr uint32_t idesc = idesc_bf16(BM, BN);
        for (int i = 0; i < niter; i++) {
            const int s = i % STAGES;
            if (!mbar_wait(&full[s], (i / STAGES) & 1)) {
                atomicOr(bad, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = smem_u32(base + s * STAGE_BYTES);
            const uint32_t a_hi = sa, a_lo = sa + A_BYTES, b_hi = sa + 2 * A_BYTES, b_lo = b_hi + B_BYTES;
#pragma unroll
            for (int kk = 0; kk < KC / 16; kk++) {
                const uint32_t o = kk * 32;  // 16 bf16 along the swizzled 128-byte row
                mma_bf16(tmem, sw128_desc(a_hi + o), sw128_desc(b_hi + o), idesc, (i | kk) != 0);
                mma_bf16(tmem, sw128_desc(a_hi + o), sw128_desc(b_lo + o), idesc, 1);
                mma_bf16(tmem, sw128_desc(a_lo + o), sw128_desc(b_hi + o), idesc, 1);
            }
            mma_commit(&empty[s]);  // stage reusable once these MMAs have read it
        }
        mma_commit(done);
    }
    __syncwarp();
    // accumulator complete?  (one waiter; the verdict is shared so that the
    // warp-collective TMEM loads below run uniformly or not at all)
    if (tid == 0 && !mbar_wait(done, 0)) atomicOr(bad, 1);
    __syncthreads();
    const bool good = (*reinterpret_cast<volatile int *>(bad) == 0);
    if (!good) {
        // a pipeline wait ran out (not expected): the tile's outputs become NaN
        // and the per-device word keeps the event.  Before the shared memory
        // and TMEM are released, the loads already issued must have landed and
        // the MMAs already issued must have finished (waits bounded as well).
        if (tid == 0) {
            for (int i = issued > STAGES ? issued - STAGES : 0; i < issued; i++)
                mbar_wait(&full[i % STAGES], (i / STAGES) & 1);
            mbar_wait(done, 0);
            atomicOr(P.status, 2);
            atomicOr(&g_timeouts, 1);
        }
        for (int u = tid; u < BM * BN; u += kThreads) {
            const int64_t ox = (int64_t)q * BM + (u % BM), oy = oy0 + u / BM;
            if (ox < P.out2 && oy < P.out1) P.y[oz * P.ys0 + oy * P.ys1 + ox] = __int_as_float(0x7fc00000);
        }
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (good) {
        const int m = warp * 32 + lane;  // TMEM lane = output along the contiguous axis
        const int64_t ox = (int64_t)q * BM + m;
        float *yrow = P.y + oz * P.ys0 + ox;
#pragma unroll
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + c0, v);
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const int64_t oy = oy0 + c0 + j;
                if (ox < P.out2 && oy < P.out1) yrow[oy * P.ys1] = v[j];
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
    }
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

// Which problems the split path takes (f32; unit stride along the middle
// axis; all index ranges within the TMA coordinate range).
bool applies(const Plan3 &P) {
    const AxisGeom *A = P.ax;
    if (P.dtype != NDCONV_F32) return false;
    if (A[1].s != 1) return false;
    for (int a = 0; a < 3; a++)
        if (A[a].L > (1 << 30) || A[a].out < 1) return false;
    return (int64_t)A[0].K * A[1].K * BM < (1 << 30);
}

}  // namespace bf16x3
}  // namespace ndconv

using namespace ndconv;
using namespace ndconv::bf16x3;

extern "C" int ndconv_conv_bf16x3(const ndconv_problem *p, const void *data, const void *kernel, void *out,
                                  void *stream) {
    Plan3 P;
    int s = plan_problem(p, 0, &P);
    if (s) return s;
    if (!data || !kernel || !out) return ndconv_fail(NDCONV_ERR_INVALID, "null pointer");
    if (!applies(P)) return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "3xBF16 path: f32 with unit middle-axis stride only");
    cudaStream_t st = (cudaStream_t)stream;
    const AxisGeom *A = P.ax;
    const Geom3<float> g = P.geom<float>();
    const int64_t Cpad = ((BM - 1) * A[2].s + (A[2].K - 1) * A[2].d + 1 + KC - 1) / KC * KC;
    const int64_t W = (A[2].L + 7) / 8 * 8;  // row pitch (16-byte multiple)
    const int64_t L = A[0].K * A[1].K;
    const size_t nX = (size_t)(A[0].L * A[1].L * W), nT = (size_t)(L * BM * Cpad);
    unsigned char *ws = nullptr;
    const size_t bytes = 2 * sizeof(__nv_bfloat16) * (nX + nT) + 256;
    NDCONV_CUDA_OK(cudaMallocAsync((void **)&ws, bytes, st));
    __nv_bfloat16 *xh = reinterpret_cast<__nv_bfloat16 *>(ws), *xl = xh + nX, *th = xl + nX, *tl = th + nT;
    int *status = reinterpret_cast<int *>(tl + nT);
    status = reinterpret_cast<int *>((reinterpret_cast<uintptr_t>(status) + 15) & ~(uintptr_t)15);
    auto fail = [&](int code) {
        cudaFreeAsync(ws, st);
        return code;
    };
    // 64-row tiles, or 32 when 64 would give fewer than two CTAs per SM
    const int64_t nseg = (A[2].out + BM - 1) / BM;
    int BN = (nseg * ((A[1].out + 63) / 64) * A[0].out < 2 * 152) ? 32 : 64;
    const int want_bn = ndconv_tune(NDCONV_TUNE_BF16X3_BN);  // the autotuner's choice
    if (want_bn == 32 || want_bn == 64) BN = want_bn;
    CUtensorMap mAh, mAl, mBh, mBl;
    {
        const cuuint64_t dA[2] = {(cuuint64_t)Cpad, (cuuint64_t)(L * BM)};
        const cuuint64_t sA[1] = {(cuuint64_t)Cpad * 2};
        const cuuint32_t bA[2] = {KC, BM};
        const cuuint64_t dB[3] = {(cuuint64_t)W, (cuuint64_t)A[1].L, (cuuint64_t)A[0].L};
        const cuuint64_t sB[2] = {(cuuint64_t)W * 2, (cuuint64_t)(W * A[1].L * 2)};
        const cuuint32_t bB[3] = {KC, (cuuint32_t)BN, 1};
        if ((s = make_map(&mAh, th, 2, dA, sA, bA)) || (s = make_map(&mAl, tl, 2, dA, sA, bA)) ||
            (s = make_map(&mBh, xh, 3, dB, sB, bB)) || (s = make_map(&mBl, xl, 3, dB, sB, bB)))
            return fail(s);
    }
    cudaMemsetAsync(status, 0, sizeof(int), st);
    split_data_kernel<<<152 * 8, 256, 0, st>>>(static_cast<const float *>(data), g, W, xh, xl, status);
    toeplitz_kernel<<<152 * 4, 256, 0, st>>>(static_cast<const float *>(kernel), g, P.reverse, Cpad, th, tl, status);
    ndconv_count_launch(2);
    Params Q{};
    Q.out0 = A[0].out;
    Q.out1 = A[1].out;
    Q.out2 = A[2].out;
    Q.s0 = A[0].s;
    Q.d0 = A[0].d;
    Q.d1 = A[1].d;
    Q.K0 = (int)A[0].K;
    Q.K1 = (int)A[1].K;
    Q.nchunk = (int)(Cpad / KC);
    Q.nseg = (int)((A[2].out + BM - 1) / BM);
    Q.s2 = A[2].s;
    Q.y = static_cast<float *>(out);
    Q.ys0 = A[1].out * A[2].out;
    Q.ys1 = A[2].out;
    Q.status = status;
    Q.dp = P.direct<float>();
    Q.x = static_cast<const float *>(data);
    Q.k = static_cast<const float *>(kernel);
    const int64_t gx = (int64_t)Q.nseg * ((A[1].out + BN - 1) / BN);
    if (gx > 0x7fffffff || A[0].out > 65535) return fail(ndconv_fail(NDCONV_ERR_UNSUPPORTED, "grid too large"));
    const void *fn = BN == 32 ? (const void *)conv_kernel<32> : (const void *)conv_kernel<64>;
    const int smem = BN == 32 ? Tile<32>::SMEM_BYTES : Tile<64>::SMEM_BYTES;
    cudaError_t e = ndconv_allow_smem(fn, smem);
    if (e != cudaSuccess) return fail(ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e)));
    const dim3 grid((unsigned)gx, (unsigned)A[0].out);
    if (BN == 32) conv_kernel<32><<<grid, kThreads, smem, st>>>(mAh, mAl, mBh, mBl, Q);
    else conv_kernel<64><<<grid, kThreads, smem, st>>>(mAh, mAl, mBh, mBl, Q);
    ndconv_count_launch();
    e = cudaGetLastError();
    cudaFreeAsync(ws, st);  // stream-ordered: after the launch has finished with it
    if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
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
