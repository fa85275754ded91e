// The persistent batch kernel and its plan (ndconv_batch_*), the FFT
// processor object and the per-instance cost model (ndconv_plan_info).
#include "fft_kernels.cuh"

// ----------------------------------------------------- processor object --
extern "C" int ndconv_fft_processor_create(int32_t dtype, ndconv_fft_processor **out) {
    if (!out) return ndconv_fail(NDCONV_ERR_INVALID, "null output pointer");
    if (dtype != NDCONV_F32 && dtype != NDCONV_F64 && dtype != NDCONV_C32 && dtype != NDCONV_C64)
        return ndconv_fail(NDCONV_ERR_UNSUPPORTED, "FFT processor needs f32/f64/c32/c64");
    auto *p = new ndconv_fft_processor{};
    p->dtype = dtype;
    cudaGetDevice(&p->device);
    *out = p;
    return NDCONV_OK;
}

extern "C" int ndconv_fft_processor_destroy(ndconv_fft_processor *p) {
    if (!p) return NDCONV_OK;
    if (p->ws || p->kbuf) cudaDeviceSynchronize();
    if (p->ws) cudaFree(p->ws);
    if (p->kbuf) cudaFree(p->kbuf);
    delete p;
    return NDCONV_OK;
}

int64_t ndconv_proc_origin_len(const ndconv_fft_processor *p) { return p->rp_origin_len; }
int32_t ndconv_proc_dtype(const ndconv_fft_processor *p) { return p->dtype; }

// ======================================================== batch plan ====
// A heterogeneous batch (instances with different shapes, kernels, modes,
// algorithms) executed by one persistent kernel.  Every instance becomes
// CTA-sized tasks: direct-convolution tiles, or the passes of its FFT
// convolution (one "level" per pass).  Tasks are stored in ticket order:
// all FFT tasks level-major across instances, then the direct tiles.  A CTA
// takes the next ticket, waits (bounded) until the previous level of the
// same instance has completed, runs the task and bumps its level counter.
// A task only waits for tasks with smaller tickets, which running CTAs have
// already claimed, so the queue always makes progress.
#include "direct_blocks.cuh"
#include "fold.h"
#include "fold_blocks.cuh"
#include "geometry.h"

namespace ndconv {
namespace batch {

enum TaskKind : int32_t {
    TK_DIRECT_SW = 1,
    TK_DIRECT_TILE4 = 2,
    TK_DIRECT_TILE1 = 3,
    TK_DIRECT_NAIVE = 4,
    TK_ROW_FWD_DATA = 10,
    TK_ROW_FWD_KERNEL = 11,
    TK_ROW_INV_OUT = 12,
    TK_ROW_FUSED = 13,
    TK_ROW_INV_MAC = 14,
    TK_COL = 20,
    TK_FOLD_SCAN = 30,  // axis-folding form: non-finite scan, chunk bx
    TK_FOLD_F1 = 31,    // first folded axis, chunk bx
    TK_FOLD_F0 = 32,    // second folded axis, chunk bx
    TK_FOLD_GEMM = 33,  // GEMM tile (bx, by)
};

// one instance of the axis-folding form inside the queue
struct FoldTaskArgs {
    FoldParams F;
    const float *x, *k;
    float *y, *W, *T1;
    int flag;  // index of its non-finite flag among the queue counters
    DirectParams<float> fb;
};
constexpr int64_t kFoldChunk = 256 * 8;  // elements per weight-folding / scan task

struct Task {
    int32_t kind, arg;
    int32_t bx, by, bz;
    int32_t done_ctr;   // counter bumped when done (-1: none)
    int32_t wait_ctr;   // counter to wait for (-1: none)
    int32_t wait_need;  // value it must reach
};

constexpr int kSpinLimit = 1 << 24;  // default poll bound: ~1-2 s of polling before giving up

__device__ __forceinline__ int ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// After the queue: instances whose skipped taps hold a non-finite weight
// get NaN everywhere, like the reference's sums.
__global__ void __launch_bounds__(256) batch_fixup_kernel(const DirectParams<float> *__restrict__ dargs,
                                                          const int *__restrict__ fix) {
    const DirectParams<float> &P = dargs[fix[blockIdx.y]];
    dead_tap_fixup_block<float>(P.k1, P.y1, P, blockIdx.x, gridDim.x);
}

// a separate function so that the GEMM tile's registers do not raise the
// other task kinds' register pressure
__device__ __noinline__ void fold_gemm_task(const FoldTaskArgs *A, int bx, int by, int *ctrs, unsigned char *smem) {
    foldk::gemm_tile<float>(A->x, A->W, A->y, A->F, ctrs + A->flag, A->k, A->fb, bx, by, smem, true);
}

__global__ void __launch_bounds__(256) persistent_kernel(const Task *__restrict__ tasks, int ntasks,
                                                         const RowArgs<float> *__restrict__ rargs,
                                                         const ColArgs<c32> *__restrict__ cargs,
                                                         const DirectParams<float> *__restrict__ dargs,
                                                         const FoldTaskArgs *__restrict__ fargs,
                                                         int *ctrs, int *ticket, int *status,
                                                         const int *poll_limit) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_ticket;
    for (;;) {
        if (threadIdx.x == 0) s_ticket = atomicAdd(ticket, 1);
        __syncthreads();
        const int t = s_ticket;
        __syncthreads();
        if (t >= ntasks) return;
        const Task tk = tasks[t];
        if (tk.wait_ctr >= 0) {
            if (threadIdx.x == 0) {
                int it = 0;
                while (ld_acquire(ctrs + tk.wait_ctr) < tk.wait_need) {
                    if (++it > *poll_limit) {
                        atomicOr(status, 1);  // dependency never completed: report, do not hang
                        break;
                    }
                    __nanosleep(64);
                }
            }
            __syncthreads();
        }
        switch (tk.kind) {
        case TK_DIRECT_SW: {
            const DirectParams<float> &P = dargs[tk.arg];
            direct_sw_block<float, 8, 16, sw_ry_max<float>()>(nullptr, nullptr, nullptr, P, tk.bx, tk.by, tk.bz,
                                                              smem_raw);
            break;
        }
        case TK_DIRECT_TILE4: {
            const DirectParams<float> &P = dargs[tk.arg];
            direct_tile_block<float, 4>(nullptr, nullptr, nullptr, P, tk.bx, tk.by, tk.bz, smem_raw);
            break;
        }
        case TK_DIRECT_TILE1: {
            const DirectParams<float> &P = dargs[tk.arg];
            direct_tile_block<float, 1>(nullptr, nullptr, nullptr, P, tk.bx, tk.by, tk.bz, smem_raw);
            break;
        }
        case TK_DIRECT_NAIVE: {
            const DirectParams<float> &P = dargs[tk.arg];
            direct_naive_range<float>(P, (int64_t)tk.bx * 256 + threadIdx.x);
            break;
        }
        case TK_ROW_FWD_DATA: row_block<float, ROW_FWD_DATA>(rargs[tk.arg], tk.bx, 0, smem_raw); break;
        case TK_ROW_FWD_KERNEL: row_block<float, ROW_FWD_KERNEL>(rargs[tk.arg], tk.bx, 0, smem_raw); break;
        case TK_ROW_INV_OUT: row_block<float, ROW_INV_OUT>(rargs[tk.arg], tk.bx, 0, smem_raw); break;
        case TK_ROW_FUSED: row_block<float, ROW_FUSED>(rargs[tk.arg], tk.bx, 0, smem_raw); break;
        case TK_ROW_INV_MAC: row_block<float, ROW_INV_MAC>(rargs[tk.arg], tk.bx, 0, smem_raw); break;
        case TK_COL: {
            const ColArgs<c32> &A = cargs[tk.arg];
            col_block<c32>(A, tk.bx, tk.by, A.n_outer, 0, smem_raw);
            break;
        }
        case TK_FOLD_SCAN: {
            const FoldTaskArgs &A = fargs[tk.arg];
            const int64_t e = min((int64_t)(tk.bx + 1) * kFoldChunk, foldk::scan_count(A.F));
            bool bad = false;
            for (int64_t u = (int64_t)tk.bx * kFoldChunk + threadIdx.x; u < e; u += blockDim.x)
                bad |= foldk::scan_elem<float>(A.x, A.k, A.F, u);
            if (bad) atomicOr(ctrs + A.flag, 1);
            break;
        }
        case TK_FOLD_F1: {
            const FoldTaskArgs &A = fargs[tk.arg];
            const int64_t e = min((int64_t)(tk.bx + 1) * kFoldChunk, foldk::f1_count<float>(A.F));
            for (int64_t u = (int64_t)tk.bx * kFoldChunk + threadIdx.x; u < e; u += blockDim.x)
                foldk::f1_elem<float>(A.k, A.F, A.T1, u);
            break;
        }
        case TK_FOLD_F0: {
            const FoldTaskArgs &A = fargs[tk.arg];
            const int64_t e = min((int64_t)(tk.bx + 1) * kFoldChunk, foldk::f0_count<float>(A.F));
            for (int64_t u = (int64_t)tk.bx * kFoldChunk + threadIdx.x; u < e; u += blockDim.x)
                foldk::f0_elem<float>(A.T1, A.F, A.W, u, true);
            break;
        }
        case TK_FOLD_GEMM: fold_gemm_task(fargs + tk.arg, tk.bx, tk.by, ctrs, smem_raw); break;
        default: break;
        }
        __threadfence();  // this CTA's results visible GPU-wide before the counter moves
        __syncthreads();
        if (threadIdx.x == 0 && tk.done_ctr >= 0) atomicAdd(ctrs + tk.done_ctr, 1);
    }
}

// work estimate of one instance (for ordering direct tiles, longest first)
struct HostInst {
    int algo;        // 0 direct, 1 FFT, 2 direct on the tensor cores (3xBF16, an ordinary launch)
    int fv;          // FFT plan variant (FftVariant)
    int standalone;  // runs as ordinary launches before the persistent kernel
    int fold;        // f32 direct instance in the axis-folding form, inside the queue
    Plan3 P;
    const void *x, *k;
    void *y;
    size_t ws_off;   // workspace offset: spectra (FFT) or folded weights (direct)
    size_t ws_bytes; // direct: folded-form scratch (0: none)
    FftConvPlan<float> cp;
    ndconv_problem prob;  // the instance's descriptor (tensor-core instances)
};

}  // namespace batch
}  // namespace ndconv

struct ndconv_batch_plan {
    int device = 0;
    int64_t n = 0;
    std::vector<ndconv::batch::HostInst> inst;
    std::vector<ndconv::batch::Task> tasks;
    std::vector<ndconv::RowArgs<float>> rargs;
    std::vector<ndconv::ColArgs<c32>> cargs;
    std::vector<ndconv::DirectParams<float>> dargs;
    std::vector<ndconv::batch::FoldTaskArgs> fargs;
    std::vector<int> fix;  // direct instances with skipped taps (non-finite fix-up after the queue)
    void *d_fix = nullptr;
    int64_t graph_kernels = 0;
    int nctrs = 0;
    size_t smem = 0;
    int grid = 0;
    void *d_tasks = nullptr, *d_rargs = nullptr, *d_cargs = nullptr, *d_dargs = nullptr, *d_fargs = nullptr;
    int *d_ctrs = nullptr;  // nctrs counters, then ticket, status (reset per run), poll bound
    int stall_ctr = -1;     // a counter no task bumps (ndconv_batch_stall_one_wait)
    int64_t stall_task = -1;  // the task redirected to it, -1: none
    int32_t stall_saved = -1; // that task's own wait counter
    void *ws = nullptr;
    size_t ws_bytes = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t n_fft = 0, n_direct = 0, n_standalone = 0;
    cudaStream_t side = nullptr;  // ordinary launches beside the persistent kernel
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

namespace ndconv {
namespace batch {

constexpr size_t kBatchSmem = 100 * 1024;  // persistent kernel's shared memory (2 CTAs per SM)

template <typename V> int upload(const std::vector<V> &v, void **d) {
    const size_t bytes = sizeof(V) * (v.empty() ? 1 : v.size());
    NDCONV_CUDA_OK(cudaMalloc(d, bytes));
    if (!v.empty()) NDCONV_CUDA_OK(cudaMemcpy(*d, v.data(), sizeof(V) * v.size(), cudaMemcpyHostToDevice));
    return NDCONV_OK;
}

// Direct tiles of instance i as tasks; returns the shared memory a task needs.
size_t direct_tasks(ndconv_batch_plan *B, HostInst &h, std::vector<Task> &out) {
    DirectParams<float> D = h.P.direct<float>();
    D.xs = nullptr;
    D.ks = nullptr;
    D.ys = nullptr;
    D.x1 = static_cast<const float *>(h.x);
    D.k1 = static_cast<const float *>(h.k);
    D.y1 = static_cast<float *>(h.y);
    restrict_live_taps(D);
    permute_axes_for_tiles(D);
    const AxisGeom &A0 = D.g.ax[0], &A1 = D.g.ax[1], &A2 = D.g.ax[2];
    int kind = 0;
    int64_t gx = 0, gy = 0;
    // the queue fills the GPU with other tasks: plan for many instances
    if (plan_sw(D, 8, 1 << 20) && smem_bytes(D) <= kBatchSmem) {
        kind = TK_DIRECT_SW;
        const int64_t TXo = sw_cols_per_cta(D, 8), TYo = sw_rows_per_cta(D);
        gx = (A2.out + TXo - 1) / TXo;
        gy = (A1.out + TYo - 1) / TYo;
    } else {
        int BX, BY;
        if (plan_tile(D, 4, BX, BY) && smem_bytes(D) <= kBatchSmem) {
            kind = TK_DIRECT_TILE4;
            gx = (A2.out + (int64_t)BX * 4 - 1) / ((int64_t)BX * 4);
        } else if (plan_tile(D, 1, BX, BY) && smem_bytes(D) <= kBatchSmem) {
            kind = TK_DIRECT_TILE1;
            gx = (A2.out + BX - 1) / BX;
        } else {
            kind = TK_DIRECT_NAIVE;
        }
        if (kind != TK_DIRECT_NAIVE) gy = (A1.out + BY - 1) / BY;
    }
    const int arg = (int)B->dargs.size();
    B->dargs.push_back(D);
    if (taps_restricted(D)) B->fix.push_back(arg);
    if (kind == TK_DIRECT_NAIVE) {
        const int64_t total = A0.out * A1.out * A2.out;
        for (int64_t b = 0; b * 256 < total; b++) out.push_back(Task{kind, arg, (int32_t)b, 0, 0, -1, -1, 0});
        return 0;
    }
    for (int64_t z = 0; z < A0.out; z++)
        for (int64_t yy = 0; yy < gy; yy++)
            for (int64_t xx = 0; xx < gx; xx++)
                out.push_back(Task{kind, arg, (int32_t)xx, (int32_t)yy, (int32_t)z, -1, -1, 0});
    return smem_bytes(D);
}

}  // namespace batch
}  // namespace ndconv

namespace ndconv {
namespace batch {

// NDCONV_OK when every pass of the FFT form fits the kernels' limits
// (shared memory, grid), NDCONV_ERR_UNSUPPORTED otherwise.  Host only.
template <typename T> int fft_fits(const Geom3<T> &g, int fv) {
    using C = typename FftConvPlan<T>::C;
    FftConvPlan<T> cp;
    int s = make_conv_plan<T>(g, cp, fv);
    if (s) return s;
    return conv_fft_passes<T>(
        g, 0, cp, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0, 1, nullptr, nullptr,
        [&](RowArgs<T> &A, int) {
            int64_t grid;
            size_t sm;
            return A.n_rows > 0 ? prep_row(A, 1, grid, sm) : NDCONV_OK;
        },
        [&](ColArgs<C> &A, int) {
            int64_t gx, gy;
            size_t sm;
            return (A.n_outer > 0 && A.n_inner > 0) ? prep_col(A, gx, gy, sm) : NDCONV_OK;
        },
        [&](RowArgs<T> &A, RowArgs<T> &B, int) {
            int64_t grid;
            size_t sm;
            int r = A.n_rows > 0 ? prep_row(A, 1, grid, sm) : NDCONV_OK;
            return r ? r : (B.n_rows > 0 ? prep_row(B, 1, grid, sm) : NDCONV_OK);
        });
}

// Build the plan: per-instance tasks, spectra, device copies of everything.
// Device memory, graph, stream and events of a plan (null members skipped).
void release(ndconv_batch_plan *B) {
    if (B->exec) cudaGraphExecDestroy(B->exec);
    if (B->graph) cudaGraphDestroy(B->graph);
    cudaFree(B->d_tasks);
    cudaFree(B->d_rargs);
    cudaFree(B->d_cargs);
    cudaFree(B->d_dargs);
    cudaFree(B->d_fargs);
    cudaFree(B->d_fix);
    cudaFree(B->d_ctrs);
    cudaFree(B->ws);
    if (B->ev_fork) cudaEventDestroy(B->ev_fork);
    if (B->ev_join) cudaEventDestroy(B->ev_join);
    if (B->side) cudaStreamDestroy(B->side);
}

int create(const ndconv_problem *probs, int64_t n, const int32_t *algo, const void *const *data,
           const void *const *kernel, void *const *out, ndconv_batch_plan **outp) {
    auto *B = new ndconv_batch_plan();
    cudaGetDevice(&B->device);
    B->n = n;
    B->inst.resize((size_t)n);
    auto fail = [&](int st) {
        release(B);  // nothing of the plan has been launched yet
        delete B;
        return st;
    };
    // ---- pass 1: plans, algorithms, spectra sizes
    size_t ws = 0;
    for (int64_t i = 0; i < n; i++) {
        HostInst &h = B->inst[(size_t)i];
        const int32_t a = algo ? algo[i] : NDCONV_ALGO_FFT;
        if (a < 0 || a >= NDCONV_ALGO_COUNT)
            return fail(ndconv_fail(NDCONV_ERR_INVALID, "algo must be 0 (direct), 1 (FFT), 2 (direct, 3xBF16) or 3..6 (FFT variants)"));
        h.algo = (a == NDCONV_ALGO_DIRECT || a == NDCONV_ALGO_DIRECT_BF16X3) ? 0 : 1;
        h.fv = (a == NDCONV_ALGO_FFT_ND) ? FFTV_ND : (a == NDCONV_ALGO_FFT_RS) ? FFTV_RS
             : (a == NDCONV_ALGO_FFT_ND_POW2) ? FFTV_ND_POW2 : (a == NDCONV_ALGO_FFT_RS_POW2) ? FFTV_RS_POW2 : FFTV_AUTO;
        int s = plan_problem(&probs[i], h.algo, &h.P);
        if (s) {
            std::string m = "instance " + std::to_string(i) + ": " + ndconv_last_error();
            return fail(ndconv_fail(s, m.c_str()));
        }
        if (single_call_int(h.P.dtype)) {
            std::string m = "instance " + std::to_string(i) + ": this integer element type runs ndconv_conv only";
            return fail(ndconv_fail(NDCONV_ERR_UNSUPPORTED, m.c_str()));
        }
        if (h.algo == 1 && (h.P.dtype == NDCONV_I32))
            return fail(ndconv_fail(NDCONV_ERR_UNSUPPORTED, "integer FFT convolution is not supported"));
        h.x = data[i];
        h.k = kernel[i];
        h.y = out[i];
        h.standalone = (h.P.dtype != NDCONV_F32);
        h.fold = 0;
        h.ws_off = 0;
        h.ws_bytes = 0;
        h.prob = probs[i];
        if (a == NDCONV_ALGO_DIRECT_BF16X3 && bf16x3_applies(h.P)) {
            // the tensor-core kernel is persistent over all SMs itself: an
            // ordinary launch beside the queue (it allocates its own planes)
            h.algo = 2;
            h.standalone = 1;
            continue;
        }
        if (h.algo == 1) {
            // transforms that do not fit one CTA's shared memory: the same
            // convolution by the direct kernels (as ndconv_conv_fft does)
            int fs = NDCONV_OK;
            switch (h.P.dtype) {
            case NDCONV_F32: fs = fft_fits<float>(h.P.geom<float>(), h.fv); break;
            case NDCONV_F64: fs = fft_fits<double>(h.P.geom<double>(), h.fv); break;
            case NDCONV_C32: fs = fft_fits<c32>(h.P.geom<c32>(), h.fv); break;
            default: fs = fft_fits<c64>(h.P.geom<c64>(), h.fv); break;
            }
            if (fs == NDCONV_ERR_UNSUPPORTED) h.algo = 0;
            else if (fs) return fail(fs);
        }
        if (h.algo == 0) {
            // direct instances taken by the axis-folding form keep their
            // folded weights in the plan's workspace; f32 ones run as queue
            // tasks, others as ordinary launches
            switch (h.P.dtype) {
            case NDCONV_F32: h.ws_bytes = direct_scratch_bytes<float>(h.P.direct<float>()); break;
            case NDCONV_F64: h.ws_bytes = direct_scratch_bytes<double>(h.P.direct<double>()); break;
            case NDCONV_I32: h.ws_bytes = direct_scratch_bytes<int32_t>(h.P.direct<int32_t>()); break;
            case NDCONV_C32: h.ws_bytes = direct_scratch_bytes<c32>(h.P.direct<c32>()); break;
            default: h.ws_bytes = direct_scratch_bytes<c64>(h.P.direct<c64>()); break;
            }
            if (h.ws_bytes) {
                h.fold = !h.standalone;
                h.ws_off = ws;
                ws += (h.ws_bytes + 255) / 256 * 256;
            }
        }
        if (h.algo == 1 && !h.standalone) {
            if ((s = make_conv_plan<float>(h.P.geom<float>(), h.cp, h.fv))) return fail(s);
            h.ws_off = ws;
            ws += (sizeof(c32) * (h.cp.nK + h.cp.nS) + 255) / 256 * 256;
        }
    }
    // standalone FFT instances of other types get their own slice as scratch
    for (int64_t i = 0; i < n; i++) {
        HostInst &h = B->inst[(size_t)i];
        if (h.algo == 1 && h.standalone) {
            h.ws_off = ws;
            size_t b = 0;
            int s = NDCONV_OK;
            // plans now, so their twiddle tables exist before any graph capture
            switch (h.P.dtype) {
            case NDCONV_F64: {
                FftConvPlan<double> cp;
                s = make_conv_plan<double>(h.P.geom<double>(), cp, h.fv);
                b = conv_fft_scratch_bytes<double>(h.P.geom<double>(), h.fv);
                break;
            }
            case NDCONV_C32: {
                FftConvPlan<c32> cp;
                s = make_conv_plan<c32>(h.P.geom<c32>(), cp, h.fv);
                b = conv_fft_scratch_bytes<c32>(h.P.geom<c32>(), h.fv);
                break;
            }
            default: {
                FftConvPlan<c64> cp;
                s = make_conv_plan<c64>(h.P.geom<c64>(), cp, h.fv);
                b = conv_fft_scratch_bytes<c64>(h.P.geom<c64>(), h.fv);
                break;
            }
            }
            if (s) return fail(s);
            ws += (b + 255) / 256 * 256;
        }
    }
    B->ws_bytes = ws;
    if (ws) {
        cudaError_t e = cudaMalloc(&B->ws, ws);
        if (e != cudaSuccess) return fail(ndconv_fail(NDCONV_ERR_NO_MEMORY, cudaGetErrorString(e)));
    }
    // ---- pass 2: FFT passes as tasks (level-major across instances)
    struct Level {
        int64_t inst;
        int ctr;
        std::vector<Task> tasks;
    };
    std::vector<std::vector<Level>> per_inst((size_t)n);
    int max_levels = 0;
    for (int64_t i = 0; i < n; i++) {
        HostInst &h = B->inst[(size_t)i];
        if (h.algo != 1 || h.standalone) continue;
        c32 *Kh = reinterpret_cast<c32 *>(static_cast<unsigned char *>(B->ws) + h.ws_off);
        c32 *S = Kh + h.cp.nK;
        std::vector<Level> &lv = per_inst[(size_t)i];
        bool too_big = false, same_level = false;
        size_t inst_smem = 0;
        auto new_level = [&]() -> Level & {
            lv.push_back(Level{i, B->nctrs++, {}});
            return lv.back();
        };
        auto emit_row = [&](RowArgs<float> &A, int cnt) -> int {
            (void)cnt;
            if (A.n_rows <= 0) return NDCONV_OK;
            int64_t grid;
            size_t sm;
            int s2 = prep_row(A, 1, grid, sm, kBatchSmem, false);
            if (s2) return s2;
            if (sm > kBatchSmem) too_big = true;
            inst_smem = std::max(inst_smem, sm);
            const int arg = (int)B->rargs.size();
            A.l2only = 1;  // producers run in the same launch: no L1-cached reads
            B->rargs.push_back(A);
            int kind = TK_ROW_FWD_DATA;
            switch (A.mode) {
            case ROW_FWD_DATA: kind = TK_ROW_FWD_DATA; break;
            case ROW_FWD_KERNEL: kind = TK_ROW_FWD_KERNEL; break;
            case ROW_INV_OUT: kind = TK_ROW_INV_OUT; break;
            case ROW_INV_MAC: kind = TK_ROW_INV_MAC; break;
            default: kind = TK_ROW_FUSED; break;
            }
            Level &L = same_level ? lv.back() : new_level();
            for (int64_t b = 0; b < grid; b++) L.tasks.push_back(Task{kind, arg, (int32_t)b, 0, 0, L.ctr, -1, 0});
            return NDCONV_OK;
        };
        // independent passes share one level (one counter)
        auto emit_pair = [&](RowArgs<float> &A, RowArgs<float> &B2, int cnt) -> int {
            int s2 = emit_row(A, cnt);
            if (s2) return s2;
            same_level = !lv.empty();
            s2 = emit_row(B2, cnt);
            same_level = false;
            return s2;
        };
        auto emit_col = [&](ColArgs<c32> &A, int cnt) -> int {
            (void)cnt;
            if (A.n_outer <= 0 || A.n_inner <= 0) return NDCONV_OK;
            int64_t gx, gy;
            size_t sm;
            int s2 = prep_col(A, gx, gy, sm);
            if (s2) return s2;
            if (sm > kBatchSmem) too_big = true;
            inst_smem = std::max(inst_smem, sm);
            const int arg = (int)B->cargs.size();
            B->cargs.push_back(A);
            Level &L = new_level();
            for (int64_t o = 0; o < A.n_outer; o++)
                for (int64_t b = 0; b < gx; b++)
                    L.tasks.push_back(Task{TK_COL, arg, (int32_t)b, (int32_t)o, 0, L.ctr, -1, 0});
            return NDCONV_OK;
        };
        const Geom3<float> g = h.P.geom<float>();
        int s = conv_fft_passes<float>(g, h.P.reverse, h.cp, static_cast<const float *>(h.x),
                                       static_cast<const float *>(h.k), static_cast<float *>(h.y), nullptr,
                                       nullptr, nullptr, 0, 1, Kh, S, emit_row, emit_col, emit_pair);
        if (s) return fail(s);
        if (too_big) {
            // does not fit the persistent kernel's shared memory: ordinary launches
            h.standalone = 1;
            lv.clear();
            continue;
        }
        B->smem = std::max(B->smem, inst_smem);
        for (size_t l = 1; l < lv.size(); l++)
            for (Task &t : lv[l].tasks) {
                t.wait_ctr = lv[l - 1].ctr;
                t.wait_need = (int32_t)lv[l - 1].tasks.size();
            }
        max_levels = std::max(max_levels, (int)lv.size());
        B->n_fft++;
    }
    // ---- axis-folding instances: scan and first folding (level 0), second
    // folding (level 1), GEMM tiles (level 2)
    for (int64_t i = 0; i < n; i++) {
        HostInst &h = B->inst[(size_t)i];
        if (!h.fold) continue;
        DirectParams<float> full = h.P.direct<float>();
        full.xs = nullptr;
        full.ks = nullptr;
        full.ys = nullptr;
        full.x1 = static_cast<const float *>(h.x);
        full.k1 = static_cast<const float *>(h.k);
        full.y1 = static_cast<float *>(h.y);
        DirectParams<float> D = full;
        restrict_live_taps(D);
        FoldTaskArgs fa;
        if (!plan_fold(D, fa.F)) return fail(ndconv_fail(NDCONV_ERR_INVALID, "axis-folding plan changed"));
        const FoldParams &F = fa.F;
        fa.x = full.x1;
        fa.k = full.k1;
        fa.y = full.y1;
        fa.W = reinterpret_cast<float *>(static_cast<unsigned char *>(B->ws) + h.ws_off);
        fa.T1 = fa.W + F.cout * F.cin * F.km;
        {
            // tap tables, built here once and copied behind the folded weights
            int32_t *dtab = reinterpret_cast<int32_t *>(fa.T1 + F.km * F.ax[F.f0].K * F.ax[F.f1].out * F.ax[F.f1].n);
            const AxisGeom &G0 = F.ax[F.f0], &G1 = F.ax[F.f1];
            const int64_t e0 = fold_table_entries(G0), e1 = fold_table_entries(G1);
            std::vector<int32_t> tab((size_t)(e0 + e1));
            for (int64_t o = 0; o < G0.out; o++)
                fold_table_row(G0, o, tab.data() + o * (G0.n + 1), tab.data() + G0.out * (G0.n + 1) + o * G0.K);
            for (int64_t o = 0; o < G1.out; o++)
                fold_table_row(G1, o, tab.data() + e0 + o * (G1.n + 1), tab.data() + e0 + G1.out * (G1.n + 1) + o * G1.K);
            cudaError_t ce = cudaMemcpy(dtab, tab.data(), sizeof(int32_t) * tab.size(), cudaMemcpyHostToDevice);
            if (ce != cudaSuccess) return fail(ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(ce)));
            fold_set_tables(fa.F, dtab);
        }
        fa.flag = B->nctrs++;
        fa.fb = full;
        const int arg = (int)B->fargs.size();
        B->fargs.push_back(fa);
        std::vector<Level> &lv = per_inst[(size_t)i];
        auto chunks = [](int64_t cnt) { return (cnt + kFoldChunk - 1) / kFoldChunk; };
        lv.push_back(Level{i, B->nctrs++, {}});
        for (int64_t b = 0; b < chunks(foldk::scan_count(F)); b++)
            lv.back().tasks.push_back(Task{TK_FOLD_SCAN, arg, (int32_t)b, 0, 0, lv.back().ctr, -1, 0});
        for (int64_t b = 0; b < chunks(foldk::f1_count<float>(F)); b++)
            lv.back().tasks.push_back(Task{TK_FOLD_F1, arg, (int32_t)b, 0, 0, lv.back().ctr, -1, 0});
        lv.push_back(Level{i, B->nctrs++, {}});
        for (int64_t b = 0; b < chunks(foldk::f0_count<float>(F)); b++)
            lv.back().tasks.push_back(Task{TK_FOLD_F0, arg, (int32_t)b, 0, 0, lv.back().ctr, -1, 0});
        lv.push_back(Level{i, B->nctrs++, {}});
        const int64_t gx = (F.ax[F.m].out + foldk::FBM - 1) / foldk::FBM, gy = (F.cout + foldk::FBN - 1) / foldk::FBN;
        for (int64_t by = 0; by < gy; by++)
            for (int64_t bx = 0; bx < gx; bx++)
                lv.back().tasks.push_back(Task{TK_FOLD_GEMM, arg, (int32_t)bx, (int32_t)by, 0, lv.back().ctr, -1, 0});
        for (size_t l = 1; l < lv.size(); l++)
            for (Task &t : lv[l].tasks) {
                t.wait_ctr = lv[l - 1].ctr;
                t.wait_need = (int32_t)lv[l - 1].tasks.size();
            }
        max_levels = std::max(max_levels, (int)lv.size());
        B->smem = std::max(B->smem, foldk::gemm_smem<float>());
        B->n_direct++;
    }
    // ---- direct tiles, largest instances first, with a work estimate per task
    std::vector<std::pair<double, int64_t>> order;
    for (int64_t i = 0; i < n; i++) {
        HostInst &h = B->inst[(size_t)i];
        if (h.algo != 0 || h.standalone || h.fold) continue;
        const AxisGeom *A = h.P.ax;
        const double work = (double)(A[0].out * A[1].out * A[2].out) * (double)(A[0].K * A[1].K * A[2].K);
        order.push_back({-work, i});
    }
    std::sort(order.begin(), order.end());
    std::vector<Task> dtasks;
    std::vector<double> dwork;
    for (auto &o : order) {
        HostInst &h = B->inst[(size_t)o.second];
        const size_t before = dtasks.size();
        B->smem = std::max(B->smem, direct_tasks(B, h, dtasks));
        const size_t cnt = dtasks.size() - before;
        for (size_t t = 0; t < cnt; t++) dwork.push_back(-o.first / (double)(cnt ? cnt : 1));
        B->n_direct++;
    }
    // ---- queue order.  A task of FFT level l > 0 spins until level l - 1 of
    // its instance is done, so levels are separated by slices of direct work
    // (which never waits): the costliest direct tiles first (they set the
    // critical path), then level 0, a slice of direct tiles, level 1, ...
    {
        double total = 0;
        for (double w : dwork) total += w;
        size_t d = 0;
        double done = 0;
        auto take = [&](double upto) {
            while (d < dtasks.size() && done < upto) {
                B->tasks.push_back(dtasks[d]);
                done += dwork[d];
                d++;
            }
        };
        take(max_levels > 0 ? 0.25 * total : total);
        for (int l = 0; l < max_levels; l++) {
            for (int64_t i = 0; i < n; i++) {
                std::vector<Level> &lv = per_inst[(size_t)i];
                if ((int)lv.size() > l) B->tasks.insert(B->tasks.end(), lv[l].tasks.begin(), lv[l].tasks.end());
            }
            take(0.25 * total + 0.75 * total * (double)(l + 1) / (double)max_levels);
        }
        take(total * 2 + 1);
    }
    for (auto &h : B->inst) B->n_standalone += h.standalone;
    // ---- device copies
    int s;
    if ((s = upload(B->tasks, &B->d_tasks)) || (s = upload(B->rargs, &B->d_rargs)) ||
        (s = upload(B->cargs, &B->d_cargs)) || (s = upload(B->dargs, &B->d_dargs)) ||
        (s = upload(B->fargs, &B->d_fargs)) || (s = upload(B->fix, &B->d_fix)))
        return fail(s);
    {
        B->stall_ctr = B->nctrs++;
        cudaError_t e = cudaMalloc((void **)&B->d_ctrs, sizeof(int) * (size_t)(B->nctrs + 3));
        if (e != cudaSuccess) return fail(ndconv_fail(NDCONV_ERR_NO_MEMORY, cudaGetErrorString(e)));
        const int lim = kSpinLimit;
        e = cudaMemcpy(B->d_ctrs + B->nctrs + 2, &lim, sizeof(int), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e)));
    }
    if (B->smem < 16) B->smem = 16;
    if (B->smem > kBatchSmem) return fail(ndconv_fail(NDCONV_ERR_INVALID, "batch task shared memory above the cap"));
    {
        cudaError_t e = ndconv_allow_smem((const void *)persistent_kernel, (int)kBatchSmem);
        if (e != cudaSuccess) return fail(ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e)));
        int per_sm = 0, sms = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persistent_kernel, 256, B->smem);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, B->device);
        if (e != cudaSuccess) return fail(ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e)));
        B->grid = std::max(1, per_sm) * sms;
        if ((int64_t)B->grid > (int64_t)B->tasks.size()) B->grid = (int)std::max<size_t>(1, B->tasks.size());
    }
    if (B->n_standalone > 0) {
        cudaError_t e = cudaStreamCreateWithFlags(&B->side, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B->ev_fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B->ev_join, cudaEventDisableTiming);
        if (e != cudaSuccess) return fail(ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e)));
    }
    *outp = B;
    return NDCONV_OK;
}

// Instances that run as ordinary launches (other element types, or FFT
// passes too large for the persistent kernel), on stream st.
int run_standalone(ndconv_batch_plan *B, cudaStream_t st) {
    for (auto &h : B->inst) {
        if (!h.standalone) continue;
        unsigned char *scr = static_cast<unsigned char *>(B->ws) + h.ws_off;
        int s = NDCONV_OK;
        if (h.algo == 2) {
            if ((s = ndconv_conv_bf16x3(&h.prob, h.x, h.k, h.y, st))) return s;
            continue;
        }
        if (h.algo == 0) {
            cudaError_t e = cudaSuccess;
            void *ds = h.ws_bytes ? scr : nullptr;
            const size_t db = h.ws_bytes;
            switch (h.P.dtype) {
            case NDCONV_F32: e = direct_conv_launch<float>((const float *)h.x, (const float *)h.k, (float *)h.y, h.P.direct<float>(), st, 0, ds, db); break;
            case NDCONV_F64: e = direct_conv_launch<double>((const double *)h.x, (const double *)h.k, (double *)h.y, h.P.direct<double>(), st, 0, ds, db); break;
            case NDCONV_I32: e = direct_conv_launch<int32_t>((const int32_t *)h.x, (const int32_t *)h.k, (int32_t *)h.y, h.P.direct<int32_t>(), st, 0, ds, db); break;
            case NDCONV_C32: e = direct_conv_launch<c32>((const c32 *)h.x, (const c32 *)h.k, (c32 *)h.y, h.P.direct<c32>(), st, 0, ds, db); break;
            default: e = direct_conv_launch<c64>((const c64 *)h.x, (const c64 *)h.k, (c64 *)h.y, h.P.direct<c64>(), st, 0, ds, db); break;
            }
            if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
            continue;
        }
        switch (h.P.dtype) {
        case NDCONV_F32: {
            const size_t b = sizeof(c32) * (h.cp.nK + h.cp.nS) + 256;
            s = conv_fft_run<float>(h.P.geom<float>(), h.P.reverse, (const float *)h.x, (const float *)h.k, (float *)h.y, nullptr, st, scr, b, h.fv);
            break;
        }
        case NDCONV_F64: s = conv_fft_run<double>(h.P.geom<double>(), h.P.reverse, (const double *)h.x, (const double *)h.k, (double *)h.y, nullptr, st, scr, conv_fft_scratch_bytes<double>(h.P.geom<double>(), h.fv), h.fv); break;
        case NDCONV_C32: s = conv_fft_run<c32>(h.P.geom<c32>(), h.P.reverse, (const c32 *)h.x, (const c32 *)h.k, (c32 *)h.y, nullptr, st, scr, conv_fft_scratch_bytes<c32>(h.P.geom<c32>(), h.fv), h.fv); break;
        default: s = conv_fft_run<c64>(h.P.geom<c64>(), h.P.reverse, (const c64 *)h.x, (const c64 *)h.k, (c64 *)h.y, nullptr, st, scr, conv_fft_scratch_bytes<c64>(h.P.geom<c64>(), h.fv), h.fv); break;
        }
        if (s) return s;
    }
    return NDCONV_OK;
}

// One execution: reset the queue, standalone instances, persistent kernel.
int enqueue(ndconv_batch_plan *B, cudaStream_t st) {
    NDCONV_CUDA_OK(cudaMemsetAsync(B->d_ctrs, 0, sizeof(int) * (size_t)(B->nctrs + 2), st));
    // ordinary launches (other element types, folded and oversized instances)
    // on a side stream, forked from and joined back into st, so they run
    // beside the persistent kernel instead of before it
    const bool side = B->n_standalone > 0 && B->side && B->ev_fork && B->ev_join;
    if (side) {
        NDCONV_CUDA_OK(cudaEventRecord(B->ev_fork, st));
        NDCONV_CUDA_OK(cudaStreamWaitEvent(B->side, B->ev_fork, 0));
    }
    int s = run_standalone(B, side ? B->side : st);
    if (s) return s;
    if (side) NDCONV_CUDA_OK(cudaEventRecord(B->ev_join, B->side));
    if (!B->tasks.empty()) {
        persistent_kernel<<<B->grid, 256, B->smem, st>>>(
            (const Task *)B->d_tasks, (int)B->tasks.size(), (const RowArgs<float> *)B->d_rargs,
            (const ColArgs<c32> *)B->d_cargs, (const DirectParams<float> *)B->d_dargs,
            (const FoldTaskArgs *)B->d_fargs, B->d_ctrs, B->d_ctrs + B->nctrs, B->d_ctrs + B->nctrs + 1,
            B->d_ctrs + B->nctrs + 2);
        ndconv_count_launch();
        NDCONV_CUDA_OK(cudaGetLastError());
    }
    if (side) NDCONV_CUDA_OK(cudaStreamWaitEvent(st, B->ev_join, 0));
    if (!B->fix.empty()) {
        // parts per instance: kernel rows over 8 CTAs at most
        batch_fixup_kernel<<<dim3(8, (unsigned)B->fix.size()), 256, 0, st>>>((const DirectParams<float> *)B->d_dargs,
                                                                             (const int *)B->d_fix);
        ndconv_count_launch();
        NDCONV_CUDA_OK(cudaGetLastError());
    }
    return NDCONV_OK;
}

}  // namespace batch
}  // namespace ndconv

extern "C" int ndconv_batch_create(const ndconv_problem *problems, int64_t n, const int32_t *algo,
                                   const void *const *data, const void *const *kernel, void *const *out,
                                   ndconv_batch_plan **plan) {
    if (!problems || !data || !kernel || !out || !plan || n < 0)
        return ndconv_fail(NDCONV_ERR_INVALID, "null argument or negative count");
    return ndconv::batch::create(problems, n, algo, data, kernel, out, plan);
}

extern "C" int ndconv_batch_run(ndconv_batch_plan *B, int32_t use_graph, void *stream) {
    if (!B) return ndconv_fail(NDCONV_ERR_INVALID, "null plan");
    cudaStream_t st = (cudaStream_t)stream;
    if (!use_graph) return ndconv::batch::enqueue(B, st);
    if (!B->exec) {
        // capture once on a private stream, replay with cudaGraphLaunch
        cudaStream_t cs;
        NDCONV_CUDA_OK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        int s = NDCONV_OK;
        const uint64_t before = ndconv_kernel_launches();
        if (e == cudaSuccess) s = ndconv::batch::enqueue(B, cs);
        B->graph_kernels = (int64_t)(ndconv_kernel_launches() - before);
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(cs, &g);
        cudaStreamDestroy(cs);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        if (s) {
            cudaGraphDestroy(g);
            return s;
        }
        e = cudaGraphInstantiate(&B->exec, g, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
        }
        B->graph = g;
    }
    NDCONV_CUDA_OK(cudaGraphLaunch(B->exec, st));
    ndconv_count_launch((uint64_t)B->graph_kernels);  // the graph's kernels run again
    return NDCONV_OK;
}

extern "C" int ndconv_batch_run_plain(ndconv_batch_plan *B, void *stream) {
    // the plain drop-in: every instance through its own per-instance entry point
    if (!B) return ndconv_fail(NDCONV_ERR_INVALID, "null plan");
    cudaStream_t st = (cudaStream_t)stream;
    for (auto &h : B->inst) {
        unsigned char *scr = static_cast<unsigned char *>(B->ws) + h.ws_off;
        if (h.algo == 2) {
            const int s = ndconv_conv_bf16x3(&h.prob, h.x, h.k, h.y, st);
            if (s) return s;
            continue;
        }
        if (h.algo == 0) {
            cudaError_t e = cudaSuccess;
            switch (h.P.dtype) {
            case NDCONV_F32: e = ndconv::direct_conv_launch<float>((const float *)h.x, (const float *)h.k, (float *)h.y, h.P.direct<float>(), st, 0); break;
            case NDCONV_F64: e = ndconv::direct_conv_launch<double>((const double *)h.x, (const double *)h.k, (double *)h.y, h.P.direct<double>(), st, 0); break;
            case NDCONV_I32: e = ndconv::direct_conv_launch<int32_t>((const int32_t *)h.x, (const int32_t *)h.k, (int32_t *)h.y, h.P.direct<int32_t>(), st, 0); break;
            case NDCONV_C32: e = ndconv::direct_conv_launch<c32>((const c32 *)h.x, (const c32 *)h.k, (c32 *)h.y, h.P.direct<c32>(), st, 0); break;
            default: e = ndconv::direct_conv_launch<c64>((const c64 *)h.x, (const c64 *)h.k, (c64 *)h.y, h.P.direct<c64>(), st, 0); break;
            }
            if (e != cudaSuccess) return ndconv_fail(NDCONV_ERR_CUDA, cudaGetErrorString(e));
            continue;
        }
        int s;
        switch (h.P.dtype) {
        case NDCONV_F32: s = ndconv::conv_fft_run<float>(h.P.geom<float>(), h.P.reverse, (const float *)h.x, (const float *)h.k, (float *)h.y, nullptr, st, scr, sizeof(c32) * (h.cp.nK + h.cp.nS) + 256, h.fv); break;
        case NDCONV_F64: s = ndconv::conv_fft_run<double>(h.P.geom<double>(), h.P.reverse, (const double *)h.x, (const double *)h.k, (double *)h.y, nullptr, st, scr, ndconv::conv_fft_scratch_bytes<double>(h.P.geom<double>(), h.fv), h.fv); break;
        case NDCONV_C32: s = ndconv::conv_fft_run<c32>(h.P.geom<c32>(), h.P.reverse, (const c32 *)h.x, (const c32 *)h.k, (c32 *)h.y, nullptr, st, scr, ndconv::conv_fft_scratch_bytes<c32>(h.P.geom<c32>(), h.fv), h.fv); break;
        default: s = ndconv::conv_fft_run<c64>(h.P.geom<c64>(), h.P.reverse, (const c64 *)h.x, (const c64 *)h.k, (c64 *)h.y, nullptr, st, scr, ndconv::conv_fft_scratch_bytes<c64>(h.P.geom<c64>(), h.fv), h.fv); break;
        }
        if (s) return s;
    }
    return NDCONV_OK;
}

extern "C" int ndconv_batch_status(ndconv_batch_plan *B, void *stream) {
    if (!B) return ndconv_fail(NDCONV_ERR_INVALID, "null plan");
    int v = 0;
    NDCONV_CUDA_OK(cudaMemcpyAsync(&v, B->d_ctrs + B->nctrs + 1, sizeof(int), cudaMemcpyDeviceToHost,
                                   (cudaStream_t)stream));
    NDCONV_CUDA_OK(cudaStreamSynchronize((cudaStream_t)stream));
    if (v) return ndconv_fail(NDCONV_ERR_TIMEOUT, "a batch task waited too long for its predecessors");
    return NDCONV_OK;
}

extern "C" int ndconv_batch_set_wait_limit(ndconv_batch_plan *B, int64_t polls) {
    if (!B) return ndconv_fail(NDCONV_ERR_INVALID, "null plan");
    const int lim = polls <= 0 ? ndconv::batch::kSpinLimit : (int)std::min<int64_t>(polls, 0x7fffffff);
    NDCONV_CUDA_OK(cudaMemcpy(B->d_ctrs + B->nctrs + 2, &lim, sizeof(int), cudaMemcpyHostToDevice));
    return NDCONV_OK;
}

extern "C" int ndconv_batch_stall_one_wait(ndconv_batch_plan *B, int32_t enable) {
    if (!B) return ndconv_fail(NDCONV_ERR_INVALID, "null plan");
    if (B->stall_task < 0) {
        for (size_t t = 0; t < B->tasks.size(); t++)
            if (B->tasks[t].wait_ctr >= 0) {
                B->stall_task = (int64_t)t;
                B->stall_saved = B->tasks[t].wait_ctr;
                break;
            }
        if (B->stall_task < 0) return ndconv_fail(NDCONV_ERR_INVALID, "no task of this plan waits on another");
    }
    ndconv::batch::Task &tk = B->tasks[(size_t)B->stall_task];
    tk.wait_ctr = enable ? B->stall_ctr : B->stall_saved;
    NDCONV_CUDA_OK(cudaMemcpy(static_cast<ndconv::batch::Task *>(B->d_tasks) + B->stall_task, &tk,
                              sizeof(ndconv::batch::Task), cudaMemcpyHostToDevice));
    return NDCONV_OK;
}

extern "C" int ndconv_batch_info(const ndconv_batch_plan *B, int64_t info[8]) {
    if (!B || !info) return ndconv_fail(NDCONV_ERR_INVALID, "null argument");
    info[0] = (int64_t)B->tasks.size();
    info[1] = B->grid;
    info[2] = (int64_t)B->smem;
    info[3] = B->n_fft;
    info[4] = B->n_direct;
    info[5] = B->n_standalone;
    info[6] = (int64_t)B->ws_bytes;
    info[7] = B->nctrs;
    return NDCONV_OK;
}

extern "C" int ndconv_batch_destroy(ndconv_batch_plan *B) {
    if (!B) return NDCONV_OK;
    cudaDeviceSynchronize();
    ndconv::batch::release(B);
    delete B;
    return NDCONV_OK;
}

// ------------------------------------------------ plan facts / cost model --
// Modelled cost of one instance under each algorithm, used by the default
// dispatcher and as features of the learned one.  Rates are round numbers
// for one GB300 (FP32 FMA ~40 T/s, shared memory ~40 TB/s, HBM ~6.8 TB/s);
// the autotuner's measurements replace them where available.
// Calibration of the modelled times against GB300 timings of 22,000
// problems of the autotuner's distribution (least squares in log time):
// FFT 3.14 x the traffic model + 34.5 us per call (its several launches),
// direct 1.03 x its model + 6.4 us.
constexpr double kFftScale = 3.14, kFftCall = 34.5e-6, kDirectScale = 1.03, kDirectCall = 6.4e-6;

extern "C" int ndconv_plan_info(const ndconv_problem *p, double out[8]) {
    using namespace ndconv;
    if (!out) return ndconv_fail(NDCONV_ERR_INVALID, "null output");
    for (int i = 0; i < 8; i++) out[i] = 0;
    Plan3 P;
    int s = plan_problem(p, 0, &P);
    if (s) return s;
    const AxisGeom *A = P.ax;
    const double nout = (double)(A[0].out * A[1].out * A[2].out);
    const double nx = (double)(A[0].n * A[1].n * A[2].n);
    double taps = (double)(A[0].K * A[1].K * A[2].K);
    double sw_s = -1;  // modelled seconds of the sliding-window kernel (f32), if it applies
    double fold_macs = -1, fold_prep = 0;  // the axis-folding form's GEMM and weight folding, if it applies
    {
        // the direct kernels only loop over taps that can see data
        DirectParams<float> D = P.direct<float>();
        restrict_live_taps(D);
        taps = (double)(D.t_n[0] * D.t_n[1] * D.t_n[2]);
        FoldParams F;
        if (plan_fold(D, F)) {
            const AxisGeom *FA = F.ax;
            fold_macs = (double)FA[F.m].out * (double)F.cout * (double)F.cin * (double)F.km;
            fold_prep = (double)F.km * FA[F.f0].K * FA[F.f1].out * FA[F.f1].n * FA[F.f1].K +
                        (double)F.cout * F.cin * F.km * FA[F.f0].K;
        }
        permute_axes_for_tiles(D);
        if (plan_sw(D, 8)) sw_s = sw_cost(D, 8, 16);
    }
    const int es = (P.dtype == NDCONV_F64 || P.dtype == NDCONV_C32 || P.dtype == NDCONV_I64 || P.dtype == NDCONV_U64)
                       ? 8
                       : (P.dtype == NDCONV_C64 ? 16 : 4);
    const double bytes = es * (nx + taps + nout);
    const double macs = nout * taps * ((P.dtype == NDCONV_C32 || P.dtype == NDCONV_C64) ? 4 : 1);
    // direct, seconds: the sliding-window kernel's fitted f32 time model plus
    // its per-call overhead when that kernel applies, else a third of a 40 T
    // multiply-add/s rate; complex taps take four FMAs, and FP64 FMAs issue
    // at a small fraction of the FP32 rate on this GPU
    const bool cplx = P.dtype == NDCONV_C32 || P.dtype == NDCONV_C64;
    const bool dbl = P.dtype == NDCONV_F64 || P.dtype == NDCONV_C64;
    const double t_fma = ((sw_s >= 0) ? sw_s * (cplx ? 4 : 1) : 3.0 * macs / 40e12) * (dbl ? 32 : 1);
    out[0] = kDirectScale * ((t_fma > bytes / 6.8e12 ? t_fma : bytes / 6.8e12) + (sw_s >= 0 ? 8.5e-6 : 4e-6)) +
             kDirectCall;
    out[2] = macs;
    if (fold_macs >= 0) {
        // the direct entry point takes the axis-folding form: a gathered
        // CUDA-core GEMM (~10 T multiply-adds/s) after the weight folding
        const double cm = (P.dtype == NDCONV_C32 || P.dtype == NDCONV_C64) ? 4 : 1;
        out[0] = cm * fold_macs / 10e12 + fold_prep / 2e12 + bytes / 6.8e12 + 10e-6;
        out[2] = cm * fold_macs;
    }
    out[3] = bytes;
    // FFT: sizes, shared-memory fit, smem-traffic model
    const bool real = !(P.dtype == NDCONV_C32 || P.dtype == NDCONV_C64);
    int64_t F[3];
    for (int a = 0; a < 3; a++) F[a] = (A[a].L == 1) ? 1 : smooth_size(A[a].L, real && a == 2);
    out[4] = (double)F[0];
    out[5] = (double)F[1];
    out[6] = (double)F[2];
    const int csz = (P.dtype == NDCONV_F64 || P.dtype == NDCONV_C64) ? 16 : 8;
    const double budget = 100.0 * 1024;  // persistent kernel share
    if (integer_dtype(P.dtype)) {
        out[1] = 1e30;
        out[7] = 0;
        return NDCONV_OK;
    }
    // rows too long for one CTA: overlap-save segments of the row-spectral form
    int64_t sn = 1, sl = 0;
    int64_t M = real ? F[2] / 2 : F[2];
    bool rs = false;
    if ((double)csz * 2 * (M + 1) * 1.07 > budget) {
        bool ok = false;
        switch (P.dtype) {
        case NDCONV_F32: ok = seg_plan<float>(A[2], false, F[2], sn, sl); break;
        case NDCONV_F64: ok = seg_plan<double>(A[2], false, F[2], sn, sl); break;
        case NDCONV_C32: ok = seg_plan<c32>(A[2], false, F[2], sn, sl); break;
        default: ok = seg_plan<c64>(A[2], false, F[2], sn, sl); break;
        }
        if (!ok) {
            out[1] = 1e30;
            out[7] = 0;
            return NDCONV_OK;
        }
        out[6] = (double)F[2];
        M = real ? F[2] / 2 : F[2];
        rs = true;
    }
    for (int a = 0; a < 2; a++)
        if (!rs && F[a] > 1 && (double)csz * 2 * F[a] * 1.07 > budget) {
            out[1] = 1e30;  // columns too long for the N-d form: conv_fft runs the direct kernels
            out[7] = 0;
            return NDCONV_OK;
        }
    auto stages = [](int64_t L) {
        FftPlanDev pl;
        if (L <= 1 || !make_plan((int)L, pl)) return 0.0;
        double c = 0;
        for (int i = 0; i < pl.nst; i++) c += 1.0;
        return c;
    };
    const double H = real ? (double)(F[2] / 2 + 1) : (double)F[2];
    const double dram_base = bytes;
    if (rs && (A[0].L > 1 || A[1].L > 1 || sn > 1)) {
        // row transforms (data rows and segments, kernel rows, output rows)
        // plus the spectral tap sums through L2
        const double rows = (double)A[0].L * A[1].L * sn + (double)A[0].K * A[1].K + (double)A[0].out * A[1].out * sn;
        const double smem_bytes = rows * H * (stages(M) + 1) * 16.0;
        const double mac_bytes = (double)A[0].out * A[1].out * sn * H * (double)(A[0].K * A[1].K) * 2.0 * csz;
        const double dram = dram_base + 2.0 * (double)A[0].L * A[1].L * sn * H * csz;
        out[1] = kFftScale * (smem_bytes / 40e12 + mac_bytes / 20e12 + dram / 6.8e12) + kFftCall;
        out[7] = 1;
        return NDCONV_OK;
    }
    const double vol = (double)F[0] * F[1] * H;  // spectrum elements
    // kernel + data forward, inverse: ~3 transforms, each stage a smem round trip (16 B/elem)
    const double st = stages(M) + stages(F[1]) + stages(F[0]) + 1;
    const double smem_bytes = 3.0 * vol * st * 16.0;
    const double dram = dram_base + 4.0 * vol * csz;
    out[1] = kFftScale * (smem_bytes / 40e12 + dram / 6.8e12) + kFftCall;
    out[7] = 1;
    return NDCONV_OK;
}
