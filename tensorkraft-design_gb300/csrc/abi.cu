// abi.cu -- C ABI of libtk_heff (declared in include/tk_heff.h).
//
// Owns the CUDA context handling, device buffers and launch sequences.  All
// entry points return status codes; failures leave a message retrievable with
// tk_last_error() on the same thread.  Nothing here aborts or traps.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "tc_gemm.cuh"
#include "tk_internal.hpp"
#include "tk_plan.cuh"

namespace tk {

static thread_local std::string g_last_error;
std::atomic<int> g_fail_device_alloc{0};

void set_error(const std::string& msg) { g_last_error = msg; }

tk_status cuda_fail(const char* op, cudaError_t e) {
    set_error(std::string(op) + ": " + cudaGetErrorName(e) + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? TK_ERR_OOM : TK_ERR_CUDA;
}

tk_status ctx_stream(tk_ctx* ctx, void** out) {
    if (!ctx->stream) {
        cudaStream_t s = nullptr;
        cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_fail("context stream", e);
        ctx->stream = s;
    }
    *out = ctx->stream;
    return TK_OK;
}

tk_status ctx_dev_scratch(tk_ctx* ctx, size_t bytes, void** out) {
    if (bytes > ctx->dev_scratch_bytes) {
        if (ctx->dev_scratch) {
            if (ctx->stream) cudaStreamSynchronize((cudaStream_t)ctx->stream);
            cudaFree(ctx->dev_scratch);
            ctx->dev_scratch = nullptr;
            ctx->dev_scratch_bytes = 0;
        }
        const size_t want = std::max<size_t>(bytes + bytes / 2, 1 << 20);
        void* p = nullptr;
        cudaError_t e = dev_malloc(&p, want);
        if (e != cudaSuccess) return cuda_fail("context device scratch", e);
        ctx->dev_scratch = p;
        ctx->dev_scratch_bytes = want;
    }
    *out = ctx->dev_scratch;
    return TK_OK;
}

tk_status ctx_host_stage(tk_ctx* ctx, size_t bytes, void** out) {
    if (bytes > ctx->host_stage_bytes) {
        if (ctx->host_stage) {
            if (ctx->stream) cudaStreamSynchronize((cudaStream_t)ctx->stream);
            cudaFreeHost(ctx->host_stage);
            ctx->host_stage = nullptr;
            ctx->host_stage_bytes = 0;
        }
        const size_t want = std::max<size_t>(bytes + bytes / 2, 1 << 20);
        void* p = nullptr;
        cudaError_t e = cudaMallocHost(&p, want);
        if (e != cudaSuccess) return cuda_fail("context host staging", e);
        ctx->host_stage = p;
        ctx->host_stage_bytes = want;
    }
    *out = ctx->host_stage;
    return TK_OK;
}

bool plan_cancelled(tk_heff2_plan* p, cudaStream_t s, const char* where) {
    if (!p->cancel || __atomic_load_n(p->cancel, __ATOMIC_ACQUIRE) == 0) return false;
    cudaStreamSynchronize(s);
    set_error(std::string(where) + ": cancelled by the caller's flag");
    return true;
}

namespace {

// Switches to the context's device for the duration of a call and restores
// the caller's current device afterwards.
struct DeviceGuard {
    int prev = -1;
    bool ok = false;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        ok = (cudaSetDevice(dev) == cudaSuccess);
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};


#define TK_CUDA(op)                                  \
    do {                                             \
        cudaError_t e_ = (op);                       \
        if (e_ != cudaSuccess) return cuda_fail(#op, e_); \
    } while (0)

}  // namespace
}  // namespace tk

using namespace tk;


extern "C" {

int32_t tk_version(void) { return 1; }

void tk_debug_fail_device_alloc(int32_t countdown) {
    g_fail_device_alloc.store(countdown > 0 ? countdown : 0, std::memory_order_relaxed);
}

const char* tk_last_error(void) { return g_last_error.c_str(); }

tk_status tk_ctx_create(int32_t device, tk_ctx** out) {
    if (!out) {
        set_error("tk_ctx_create: null out");
        return TK_ERR_INVALID_ARG;
    }
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) return cuda_fail("cudaGetDeviceCount", e);
    if (device < 0 || device >= n) {
        set_error("tk_ctx_create: device index out of range");
        return TK_ERR_INVALID_ARG;
    }
    tk_ctx* c = new (std::nothrow) tk_ctx;
    if (!c) {
        set_error("tk_ctx_create: host allocation failed");
        return TK_ERR_OOM;
    }
    c->device = device;
    *out = c;
    return TK_OK;
}

void tk_ctx_destroy(tk_ctx* ctx) {
    if (!ctx) return;
    ctx_release_solver(ctx);
    {
        DeviceGuard g(ctx->device);
        if (ctx->stream) cudaStreamSynchronize((cudaStream_t)ctx->stream);
        if (ctx->dev_scratch) cudaFree(ctx->dev_scratch);
        if (ctx->host_stage) cudaFreeHost(ctx->host_stage);
        if (ctx->stream) cudaStreamDestroy((cudaStream_t)ctx->stream);
    }
    delete ctx;
}

tk_status tk_heff2_plan_create(tk_ctx* ctx, const tk_env* env_l, const tk_env* env_r, const tk_bst* w_i,
                               const tk_bst* w_j, const int32_t* psi_flux, int32_t precision,
                               tk_heff2_plan** out) {
    if (!ctx || !env_l || !env_r || !w_i || !w_j || !out) {
        set_error("tk_heff2_plan_create: null argument");
        return TK_ERR_INVALID_ARG;
    }
    return plan_create_impl(ctx, env_l, env_r, w_i, w_j, psi_flux, precision, nullptr, nullptr, out);
}

tk_status tk_heff2_plan_footprint(const tk_env* env_l, const tk_env* env_r, const tk_bst* w_i, const tk_bst* w_j,
                                  const int32_t* psi_flux, int32_t precision, int64_t* block_dim, int64_t* n_blocks,
                                  int64_t* device_bytes) {
    if (!env_l || !env_r || !w_i || !w_j) {
        set_error("tk_heff2_plan_footprint: null argument");
        return TK_ERR_INVALID_ARG;
    }
    if (precision != TK_PREC_FP64 && precision != TK_PREC_BF16X3) {
        set_error("tk_heff2_plan_footprint: unknown precision");
        return TK_ERR_INVALID_ARG;
    }
    std::string err;
    Heff2Tables H;
    tk_status st = build_heff2_tables(*env_l, *env_r, *w_i, *w_j, psi_flux, kF64TileM, kF64TileN, H, err);
    if (st == TK_OK) st = ensure_tc_tables(H, err);  // the stack sizes of both precisions come from them
    if (st != TK_OK) {
        set_error("tk_heff2_plan_footprint: " + err);
        return st;
    }
    auto vb = [](const auto& v) { return (double)v.size() * sizeof(v[0]); };
    double b = 0.0;
    {
        // the stacked FP64 operands a plan builds (its default schedule): the
        // same L, R and T2 stack rows as the split tables, in FP64, and T1 in
        // FP64 (piece tables about one entry per 64 output rows of a tile).
        // The grouped schedule's state is not counted: it is uploaded only
        // when that schedule is chosen.
        const TcTables& C = H.tc;
        b += 8.0 * kTcBK * ((double)C.lq_rows + C.rq_rows + std::max<int64_t>(C.t2q_rows, 1)) +
             8.0 * std::max<int64_t>(C.t1_total, 1) + 2.0 * (vb(C.tiles1) + vb(C.tiles3)) + vb(C.jobs) +
             vb(C.terms) + 8.0 * C.terms.size() + vb(C.yrow) + vb(C.t1col_base) + vb(C.t1col_stride) + vb(C.xsrc) +
             vb(C.xstride);
    }
    if (precision == TK_PREC_BF16X3) {
        const TcTables& C = H.tc;
        const double row = 2.0 * 2.0 * kTcBK;  // hi + lo bf16 per operand row
        b += row * ((double)C.lq_rows + C.rq_rows + C.t2q_rows + C.xq_rows) + 4.0 * std::max<int64_t>(C.t1_total, 1);
        b += vb(C.tiles1) + vb(C.tiles1x) + vb(C.tiles3) + vb(C.split) + vb(C.jobs) + vb(C.terms) + vb(C.yrow) +
             vb(C.t1col_base) + vb(C.t1col_stride) + vb(C.xsrc) + vb(C.xstride) + sizeof(int);
    }
    if (block_dim) *block_dim = H.total;
    if (n_blocks) *n_blocks = (int64_t)H.keys.size();
    if (device_bytes) *device_bytes = (int64_t)b;
    return TK_OK;
}

}  // extern "C"

// The device state of the grouped and per-block FP64 schedules (environment
// slabs, intermediates, GEMM and combine tables; for a complex plan also the
// imaginary intermediates), uploaded on the first request for one of them.
tk_status tk::ensure_grouped(tk_heff2_plan* p) {
    if (p->grouped_ready) return TK_OK;
    const Heff2Tables& H = p->host;
    DeviceGuard g(p->device);
    TK_CUDA(p->lbuf.upload(H.lbuf));
    TK_CUDA(p->rbuf.upload(H.rbuf));
    TK_CUDA(p->t1.alloc((size_t)std::max<int64_t>(H.t1_total, 1)));
    TK_CUDA(p->t2.alloc((size_t)std::max<int64_t>(H.t2_total, 1)));
    TK_CUDA(p->g1.upload(H.g1));
    TK_CUDA(p->g3.upload(H.g3));
    TK_CUDA(p->jobs.upload(H.jobs));
    TK_CUDA(p->terms.upload(H.terms));
    if (p->is_complex) {
        TK_CUDA(p->t1_im.alloc(p->t1.n));
        TK_CUDA(p->t2_im.alloc(p->t2.n));
    }
    p->grouped_ready = true;
    return TK_OK;
}

// Shared by tk_heff2_plan_create (dense host environments) and
// tk_heff2_plan_create_dev (host copies of canonical block-layout ones).
tk_status tk::plan_create_impl(tk_ctx* ctx, const tk_env* env_l, const tk_env* env_r, const tk_bst* w_i,
                               const tk_bst* w_j, const int32_t* psi_flux, int32_t precision, const double* l_blocks,
                               const double* r_blocks, tk_heff2_plan** out, bool stacked) {
    *out = nullptr;
    if (precision != TK_PREC_FP64 && precision != TK_PREC_BF16X3) {
        set_error("tk_heff2_plan_create: unknown precision");
        return TK_ERR_INVALID_ARG;
    }
    std::unique_ptr<tk_heff2_plan> p(new (std::nothrow) tk_heff2_plan);
    if (!p) {
        set_error("tk_heff2_plan_create: host allocation failed");
        return TK_ERR_OOM;
    }
    std::string err;
    tk_status st = build_heff2_tables(*env_l, *env_r, *w_i, *w_j, psi_flux, kF64TileM, kF64TileN, p->host, err,
                                      l_blocks, r_blocks);
    if (st != TK_OK) {
        set_error("tk_heff2_plan_create: " + err);
        return st;
    }
    DeviceGuard g(ctx->device);
    if (!g.ok) {
        set_error("tk_heff2_plan_create: cudaSetDevice failed");
        return TK_ERR_CUDA;
    }
    p->device = ctx->device;
    const Heff2Tables& H = p->host;
    TK_CUDA(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    // the grouped schedule's device state is uploaded when that schedule is chosen
    p->n_jobs = (int)H.jobs.size();
    p->precision = TK_PREC_FP64;
    // the FP64 matvec runs on operand stacks (TK_SCHED_STACKED); without
    // `stacked` the caller sets the schedule before the plan is used
    if (stacked) {
        tk_status s3 = tk_heff2_set_schedule(p.get(), TK_SCHED_STACKED);
        if (s3 != TK_OK) return s3;
    }
    if (precision != TK_PREC_FP64) {
        tk_status s2 = tk_heff2_set_precision(p.get(), precision);
        if (s2 != TK_OK) return s2;
    }
    *out = p.release();
    return TK_OK;
}

extern "C" {

void tk_heff2_plan_destroy(tk_heff2_plan* plan) {
    if (!plan) return;
    DeviceGuard g(plan->device);
    delete plan;
}

tk_status tk_heff2_dims(const tk_heff2_plan* plan, int64_t* dense_dim, int64_t* block_dim, int64_t* n_blocks) {
    if (!plan) {
        set_error("tk_heff2_dims: null plan");
        return TK_ERR_INVALID_ARG;
    }
    const Heff2Tables& H = plan->host;
    if (dense_dim) *dense_dim = H.d_i * H.d_j * H.d_l * H.d_r;
    if (block_dim) *block_dim = H.total;
    if (n_blocks) *n_blocks = (int64_t)H.keys.size();
    return TK_OK;
}

tk_status tk_heff2_blocks(const tk_heff2_plan* plan, uint64_t* keys, int64_t* offsets) {
    if (!plan) {
        set_error("tk_heff2_blocks: null plan");
        return TK_ERR_INVALID_ARG;
    }
    const Heff2Tables& H = plan->host;
    if (keys) std::copy(H.keys.begin(), H.keys.end(), keys);
    if (offsets) std::copy(H.blk_off.begin(), H.blk_off.end(), offsets);
    return TK_OK;
}

tk_status tk_heff2_cost(const tk_heff2_plan* plan, double* flops, double* bytes) {
    if (!plan) {
        set_error("tk_heff2_cost: null plan");
        return TK_ERR_INVALID_ARG;
    }
    const Heff2Tables& H = plan->host;
    if (flops) *flops = H.g1.flops + H.comb_flops + H.g3.flops;
    if (bytes) *bytes = H.alg_bytes;
    return TK_OK;
}

tk_status tk_heff2_set_precision(tk_heff2_plan* plan, int32_t precision) {
    if (!plan) {
        set_error("tk_heff2_set_precision: null plan");
        return TK_ERR_INVALID_ARG;
    }
    if (precision == TK_PREC_FP64) {
        plan->precision = precision;
        return TK_OK;
    }
    if (precision != TK_PREC_BF16X3) {
        set_error("tk_heff2_set_precision: unknown precision");
        return TK_ERR_INVALID_ARG;
    }
    if (plan->is_complex) {
        set_error("tk_heff2_set_precision: complex plans run in FP64 only");
        return TK_ERR_UNSUPPORTED;
    }
    DeviceGuard g(plan->device);
    if (!plan->tc) {
        std::string err;
        std::unique_ptr<TcPlan, TcPlanDeleter> tc;
        tk_status st = ensure_tc_tables(plan->host, err);
        if (st == TK_OK)
            st = guard_host("split-precision plan", err,
                            [&] { return tc_plan_create(plan->host, plan->lbuf.p, plan->rbuf.p, tc, err); });
        if (st != TK_OK) {
            set_error("tk_heff2_set_precision: " + err);
            return st;
        }
        plan->tc = std::move(tc);
    }
    plan->precision = precision;
    return TK_OK;
}

// The FP64 matvec: three stream-ordered launches.
// One launch per output block (the per-block baseline schedule).
static cudaError_t launch_per_block(const DevGemm& g, const double* A, const double* B, double* C, cudaStream_t s) {
    for (size_t t = 0; t + 1 < g.task_tile_begin.size(); ++t) {
        const int b = g.task_tile_begin[t], n = g.task_tile_begin[t + 1] - b;
        cudaError_t e = launch_gemm_f64(g.tiles_by_task.p + b, n, g.tasks.p, g.segs.p, A, B, C, s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// The FP64 matvec: three stream-ordered stages.
static tk_status apply_fp64(tk_heff2_plan* p, const double* x, double* y, cudaStream_t s) {
    if (p->schedule == TK_SCHED_STACKED) {
        TK_CUDA(f64stack_apply(*p->f64s, x, y, s));
        return TK_OK;
    }
    if (p->schedule == TK_SCHED_PER_BLOCK) {
        TK_CUDA(launch_per_block(p->g1, p->lbuf.p, x, p->t1.p, s));
        TK_CUDA(launch_combine_f64(p->jobs.p, p->n_jobs, p->terms.p, p->t1.p, p->t2.p, s));
        TK_CUDA(launch_per_block(p->g3, p->t2.p, p->rbuf.p, y, s));
        return TK_OK;
    }
    TK_CUDA(launch_gemm_f64(p->g1.tiles.p, p->g1.n_tiles, p->g1.tasks.p, p->g1.segs.p, p->lbuf.p, x, p->t1.p, s));
    TK_CUDA(launch_combine_f64(p->jobs.p, p->n_jobs, p->terms.p, p->t1.p, p->t2.p, s));
    TK_CUDA(launch_gemm_f64(p->g3.tiles.p, p->g3.n_tiles, p->g3.tasks.p, p->g3.segs.p, p->t2.p, p->rbuf.p, y, s));
    return TK_OK;
}

static int per_block_launches(const DevGemm& g) {
    int n = 0;
    for (size_t t = 0; t + 1 < g.task_tile_begin.size(); ++t) n += g.task_tile_begin[t + 1] > g.task_tile_begin[t];
    return n;
}

extern "C" tk_status tk_heff2_launches(const tk_heff2_plan* plan, int32_t* per_apply) {
    if (!plan || !per_apply) {
        set_error("tk_heff2_launches: invalid argument");
        return TK_ERR_INVALID_ARG;
    }
    const tk_heff2_plan* p = plan;
    int n = 0;
    if (p->is_complex && p->schedule == TK_SCHED_STACKED) {
        n = f64stack_launches(*p->f64s) + (p->n_jobs > 0);  // the combine runs once per part
    } else if (p->is_complex) {
        n = 4 * (p->g1.n_tiles > 0) + 2 * (p->n_jobs > 0) + 4 * (p->g3.n_tiles > 0);
    } else if (p->precision == TK_PREC_BF16X3) {
        n = tc_launches(*p->tc);
    } else if (p->schedule == TK_SCHED_STACKED) {
        n = f64stack_launches(*p->f64s);
    } else if (p->schedule == TK_SCHED_PER_BLOCK) {
        n = per_block_launches(p->g1) + (p->n_jobs > 0) + per_block_launches(p->g3);
    } else {
        n = (p->g1.n_tiles > 0) + (p->n_jobs > 0) + (p->g3.n_tiles > 0);
    }
    *per_apply = n;
    return TK_OK;
}

// The complex FP64 matvec: each stage's GEMM as four real launches over the
// same tables (planar operands); the channel combine (real MPO) on each part.
tk_status tk_heff2_apply_complex_s(tk_heff2_plan* p, const double* xr, const double* xi, double* yr, double* yi,
                                   cudaStream_t s) {
    if (!p->is_complex) {
        set_error("complex matvec on a real plan");
        return TK_ERR_INVALID_ARG;
    }
    if (p->schedule == TK_SCHED_STACKED) {
        TK_CUDA(f64stack_apply_complex(*p->f64s, xr, xi, yr, yi, s));
        return TK_OK;
    }
    TK_CUDA(launch_gemm_c64(p->g1.tiles.p, p->g1.n_tiles, p->g1.tasks.p, p->g1.segs.p, p->lbuf.p, p->lbuf_im.p, xr, xi,
                            p->t1.p, p->t1_im.p, false, s));
    TK_CUDA(launch_combine_f64(p->jobs.p, p->n_jobs, p->terms.p, p->t1.p, p->t2.p, s));
    TK_CUDA(launch_combine_f64(p->jobs.p, p->n_jobs, p->terms.p, p->t1_im.p, p->t2_im.p, s));
    TK_CUDA(launch_gemm_c64(p->g3.tiles.p, p->g3.n_tiles, p->g3.tasks.p, p->g3.segs.p, p->t2.p, p->t2_im.p, p->rbuf.p,
                            p->rbuf_im.p, yr, yi, false, s));
    return TK_OK;
}

tk_status tk_heff2_apply_complex(tk_heff2_plan* plan, const double* xr, const double* xi, double* yr, double* yi,
                                 void* stream) {
    if (!plan || ((!xr || !xi || !yr || !yi) && plan->host.total > 0)) {
        set_error("tk_heff2_apply_complex: null argument");
        return TK_ERR_INVALID_ARG;
    }
    if (plan->host.total == 0) return TK_OK;
    DeviceGuard g(plan->device);
    return tk_heff2_apply_complex_s(plan, xr, xi, yr, yi, (cudaStream_t)stream);
}

tk_status tk_heff2_set_cancel_flag(tk_heff2_plan* plan, const int32_t* flag) {
    if (!plan) {
        set_error("tk_heff2_set_cancel_flag: null plan");
        return TK_ERR_INVALID_ARG;
    }
    plan->cancel = flag;
    return TK_OK;
}

tk_status tk_heff2_inject_error_word(tk_heff2_plan* plan, int32_t code) {
    if (!plan || code == 0) {
        set_error("tk_heff2_inject_error_word: null plan or zero code");
        return TK_ERR_INVALID_ARG;
    }
    if (plan->precision != TK_PREC_BF16X3 || !plan->tc) {
        set_error("tk_heff2_inject_error_word: the plan runs no tensor-core kernels");
        return TK_ERR_UNSUPPORTED;
    }
    DeviceGuard g(plan->device);
    TK_CUDA(cudaMemcpy(tc_error_word(*plan->tc), &code, sizeof(int32_t), cudaMemcpyHostToDevice));
    return TK_OK;
}

// Rebuilds the split tables and the tensor-core plan with `o`; the cached
// CUDA graphs hold the old kernels' tables and are dropped.
static tk_status apply_tc_options(tk_heff2_plan* plan, const TcOptions& o) {
    std::string err;
    tk_status st;
    const TcOptions cur = plan->host.tcopt;
    if (plan->host.tc_built && o.tall_max_mtiles == cur.tall_max_mtiles && o.fuse_max_ntiles == cur.fuse_max_ntiles) {
        // only launch forms change (combine form, persistent or narrow stage
        // 1): the split tables and operands stay; the cached graphs go
        if (plan->tc && (st = tc_set_launch_forms(*plan->tc, o, err)) != TK_OK) {
            set_error("tc options: " + err);
            return st;
        }
        plan->host.tcopt = o;
        if (plan->host_exec) {
            cudaGraphExecDestroy(plan->host_exec);
            plan->host_exec = nullptr;
        }
        plan->lz_graph.reset();
        return TK_OK;
    }
    st = rebuild_tc_tables(plan->host, o, err);
    if (st != TK_OK) {
        set_error("tc options: " + err);
        return st;
    }
    if (plan->host_exec) {
        cudaGraphExecDestroy(plan->host_exec);
        plan->host_exec = nullptr;
    }
    plan->lz_graph.reset();
    if (plan->tc) {
        std::unique_ptr<TcPlan, TcPlanDeleter> tc;
        st = guard_host("split-precision plan", err,
                        [&] { return tc_plan_create(plan->host, plan->lbuf.p, plan->rbuf.p, tc, err); });
        if (st != TK_OK) {
            set_error("tc options: " + err);
            plan->tc.reset();
            plan->precision = TK_PREC_FP64;
            return st;
        }
        plan->tc = std::move(tc);
    }
    return TK_OK;
}

tk_status tk_heff2_set_tc_options(tk_heff2_plan* plan, const tk_tc_options* opts) {
    if (!plan || !opts || opts->tall_max_mtiles < 1 || opts->fuse_max_ntiles < 0 || opts->combine_warps < 0 ||
        opts->combine_warps > 3 || opts->stage1_persistent < 0 || opts->stage1_persistent > 1 ||
        opts->stage1_narrow < 0 || opts->stage1_narrow > 1) {
        set_error("tk_heff2_set_tc_options: invalid argument");
        return TK_ERR_INVALID_ARG;
    }
    if (plan->is_complex) {
        set_error("tk_heff2_set_tc_options: complex plans run in FP64 only");
        return TK_ERR_UNSUPPORTED;
    }
    DeviceGuard g(plan->device);
    TcOptions o;
    o.tall_max_mtiles = opts->tall_max_mtiles;
    o.fuse_max_ntiles = opts->fuse_max_ntiles;
    o.combine_warps = opts->combine_warps;
    o.stage1_persistent = opts->stage1_persistent;
    o.stage1_narrow = opts->stage1_narrow;
    return apply_tc_options(plan, o);
}

tk_status tk_heff2_get_tc_options(const tk_heff2_plan* plan, tk_tc_options* opts) {
    if (!plan || !opts) {
        set_error("tk_heff2_get_tc_options: invalid argument");
        return TK_ERR_INVALID_ARG;
    }
    opts->tall_max_mtiles = plan->host.tcopt.tall_max_mtiles;
    opts->fuse_max_ntiles = plan->host.tcopt.fuse_max_ntiles;
    opts->combine_warps = plan->host.tcopt.combine_warps;
    opts->stage1_persistent = plan->host.tcopt.stage1_persistent;
    opts->stage1_narrow = plan->host.tcopt.stage1_narrow;
    return TK_OK;
}

tk_status tk_heff2_set_schedule(tk_heff2_plan* plan, int32_t schedule) {
    if (!plan || (schedule != TK_SCHED_GROUPED && schedule != TK_SCHED_PER_BLOCK && schedule != TK_SCHED_STACKED)) {
        set_error("tk_heff2_set_schedule: invalid argument");
        return TK_ERR_INVALID_ARG;
    }
    if (schedule != TK_SCHED_STACKED) {
        tk_status st = ensure_grouped(plan);
        if (st != TK_OK) {
            set_error("tk_heff2_set_schedule: " + std::string(tk_last_error()));
            return st;
        }
    }
    if (schedule == TK_SCHED_STACKED && !plan->f64s) {
        DeviceGuard g(plan->device);
        std::string err;
        // a complex plan's imaginary slabs live on the device only: host copies for the stacks
        std::vector<double> lim, rim;
        if (plan->is_complex) {
            lim.resize(plan->lbuf_im.n);
            rim.resize(plan->rbuf_im.n);
            if (lim.size() != plan->host.lbuf.size() || rim.size() != plan->host.rbuf.size()) {
                set_error("tk_heff2_set_schedule: imaginary environment slabs of another size");
                return TK_ERR_INVALID_ARG;
            }
            if (!lim.empty()) TK_CUDA(cudaMemcpy(lim.data(), plan->lbuf_im.p, sizeof(double) * lim.size(),
                                                 cudaMemcpyDeviceToHost));
            if (!rim.empty()) TK_CUDA(cudaMemcpy(rim.data(), plan->rbuf_im.p, sizeof(double) * rim.size(),
                                                 cudaMemcpyDeviceToHost));
        }
        tk_status st = build_f64_stacks(plan->host, err, plan->is_complex ? lim.data() : nullptr,
                                        plan->is_complex ? rim.data() : nullptr);
        if (st == TK_OK)
            st = guard_host("stacked FP64 plan", err, [&] { return f64stack_create(plan->host.f64st, plan->f64s, err); });
        // the device copy is the one that runs: the host tables go
        plan->host.f64st = TcTables();
        if (st != TK_OK) {
            plan->f64s.reset();
            set_error("tk_heff2_set_schedule: " + err);
            return st;
        }
    }
    if (plan->schedule != schedule) plan->lz_graph.reset();  // captured with the old schedule's kernels
    plan->schedule = schedule;
    return TK_OK;
}

tk_status tk_heff2_get_schedule(const tk_heff2_plan* plan, int32_t* schedule) {
    if (!plan || !schedule) {
        set_error("tk_heff2_get_schedule: invalid argument");
        return TK_ERR_INVALID_ARG;
    }
    *schedule = plan->schedule;
    return TK_OK;
}

tk_status tk_heff2_apply_prec(tk_heff2_plan* p, const double* x, double* y, cudaStream_t s, int precision) {
    if (p->is_complex) {
        set_error("real matvec on a complex plan (use tk_heff2_apply_complex)");
        return TK_ERR_INVALID_ARG;
    }
    if (precision == TK_PREC_BF16X3) {
        std::string err;
        cudaError_t e = tc_apply(*p->tc, p->host, p->jobs.p, p->n_jobs, p->terms.p, x, y, s, err);
        if (e != cudaSuccess) return cuda_fail(err.c_str(), e);
        return TK_OK;
    }
    return apply_fp64(p, x, y, s);
}

tk_status tk_heff2_apply(tk_heff2_plan* plan, const double* x_dev, double* y_dev, void* stream) {
    if (!plan || (!x_dev && plan->host.total > 0) || (!y_dev && plan->host.total > 0)) {
        set_error("tk_heff2_apply: null argument");
        return TK_ERR_INVALID_ARG;
    }
    if (plan->host.total == 0) return TK_OK;
    DeviceGuard g(plan->device);
    return tk_heff2_apply_prec(plan, x_dev, y_dev, (cudaStream_t)stream, plan->precision);
}

static tk_status ensure_host_staging(tk_heff2_plan* p) {
    size_t n = (size_t)std::max<int64_t>(p->host.total, 1);
    if (!p->hx.p) TK_CUDA(p->hx.alloc(n));
    if (!p->hy.p) TK_CUDA(p->hy.alloc(n));
    if (!p->pin_x) TK_CUDA(cudaMallocHost(&p->pin_x, sizeof(double) * n));
    if (!p->pin_y) TK_CUDA(cudaMallocHost(&p->pin_y, sizeof(double) * n));
    if (!p->pin_err) {
        TK_CUDA(cudaMallocHost(&p->pin_err, sizeof(int)));
        *p->pin_err = 0;
    }
    if (!p->copy_stream) TK_CUDA(cudaStreamCreateWithFlags(&p->copy_stream, cudaStreamNonBlocking));
    if (!p->ev_fork) TK_CUDA(cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming));
    for (cudaEvent_t& e : p->ev_piece)
        if (!e) TK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return TK_OK;
}

// Split matvec from a host buffer copied in k pieces: the stage-1 tiles that
// read only the first j pieces run while the later ones are in flight (copy
// stream forked from and joined back into `s`), then the rest of the matvec
// as usual.  Stream-ordered; used inside a graph capture.
static tk_status enqueue_split_psi_pieces(tk_heff2_plan* p, const double* x, double* y, int k, const int64_t* x_cut,
                                          const int32_t* n1_cut, cudaStream_t s) {
    TK_CUDA(cudaEventRecord(p->ev_fork, s));
    TK_CUDA(cudaStreamWaitEvent(p->copy_stream, p->ev_fork, 0));
    for (int j = 0; j < k; ++j) {
        const int64_t len = x_cut[j + 1] - x_cut[j];
        if (len > 0)
            TK_CUDA(cudaMemcpyAsync(p->hx.p + x_cut[j], x + x_cut[j], sizeof(double) * len, cudaMemcpyHostToDevice,
                                    p->copy_stream));
        TK_CUDA(cudaEventRecord(p->ev_piece[j], p->copy_stream));
    }
    for (int j = 0; j < k; ++j) {
        TK_CUDA(cudaStreamWaitEvent(s, p->ev_piece[j], 0));
        if (n1_cut[j + 1] > n1_cut[j])
            TK_CUDA(tc_stage1_range(*p->tc, p->hx.p, n1_cut[j], n1_cut[j + 1] - n1_cut[j], s));
    }
    for (int stage = 1; stage < 3; ++stage) {
        std::string err;
        cudaError_t e = tc_apply_stage(*p->tc, p->host, p->jobs.p, p->n_jobs, p->terms.p, p->hx.p, y, s, stage, err);
        if (e != cudaSuccess) return cuda_fail(err.c_str(), e);
    }
    return TK_OK;
}

// Device address of page-locked, mapped host memory; nullptr for anything else.
static void* mapped_host_ptr(const void* h) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Queues the read-back of the tensor-core error word behind the matvec,
// waits for the stream once, and reports a bounded wait that ran out.
static tk_status finish_host_call(tk_heff2_plan* p, cudaStream_t s) {
    const bool tc = p->precision == TK_PREC_BF16X3;
    if (tc) TK_CUDA(cudaMemcpyAsync(p->pin_err, tc_error_word(*p->tc), sizeof(int), cudaMemcpyDeviceToHost, s));
    TK_CUDA(cudaStreamSynchronize(s));
    if (tc && *p->pin_err != 0) return tc_check_error(*p->tc, s);
    return TK_OK;
}

tk_status tk_heff2_set_psi_pieces(tk_heff2_plan* plan, int32_t pieces) {
    if (!plan || pieces < 1 || pieces > kTcPsiPieces || kTcPsiPieces % pieces != 0) {
        set_error("tk_heff2_set_psi_pieces: invalid argument");
        return TK_ERR_INVALID_ARG;
    }
    plan->psi_pieces = pieces;
    return TK_OK;
}

tk_status tk_heff2_set_host_io(tk_heff2_plan* plan, int32_t mode) {
    if (!plan || mode < TK_HOST_IO_STAGED || mode > TK_HOST_IO_AUTO) {
        set_error("tk_heff2_set_host_io: invalid argument");
        return TK_ERR_INVALID_ARG;
    }
    plan->host_io = mode;
    return TK_OK;
}

tk_status tk_heff2_dense_to_flat(const tk_heff2_plan* plan, const double* dense, double* flat) {
    if (!plan || !dense || !flat) {
        set_error("tk_heff2_dense_to_flat: null argument");
        return TK_ERR_INVALID_ARG;
    }
    const Heff2Tables& H = plan->host;
    for (const SubMap& m : H.submaps)
        for (int32_t r = 0; r < m.rows; ++r)
            std::memcpy(flat + m.flat_off + (int64_t)r * m.cols, dense + m.dense_off + (int64_t)r * H.d_r,
                        sizeof(double) * m.cols);
    return TK_OK;
}

tk_status tk_heff2_flat_to_dense(const tk_heff2_plan* plan, const double* flat, double* dense) {
    if (!plan || !dense || !flat) {
        set_error("tk_heff2_flat_to_dense: null argument");
        return TK_ERR_INVALID_ARG;
    }
    const Heff2Tables& H = plan->host;
    std::memset(dense, 0, sizeof(double) * (size_t)(H.d_i * H.d_j * H.d_l * H.d_r));
    for (const SubMap& m : H.submaps)
        for (int32_t r = 0; r < m.rows; ++r)
            std::memcpy(dense + m.dense_off + (int64_t)r * H.d_r, flat + m.flat_off + (int64_t)r * m.cols,
                        sizeof(double) * m.cols);
    return TK_OK;
}

tk_status tk_heff2_apply_host_flat(tk_heff2_plan* plan, const double* x, double* y) {
    if (!plan || !x || !y) {
        set_error("tk_heff2_apply_host_flat: null argument");
        return TK_ERR_INVALID_ARG;
    }
    const int64_t n = plan->host.total;
    if (n == 0) return TK_OK;
    DeviceGuard g(plan->device);
    tk_status st = ensure_host_staging(plan);
    if (st != TK_OK) return st;
    cudaStream_t s = plan->stream;
    int mode = plan->precision == TK_PREC_BF16X3 ? plan->host_io : TK_HOST_IO_STAGED;
    if (mode == TK_HOST_IO_AUTO) mode = TK_HOST_IO_DIRECT_OUT;
    const double* mx = static_cast<const double*>(mapped_host_ptr(x));
    double* my = static_cast<double*>(mapped_host_ptr(y));
    const double* dx = mode == TK_HOST_IO_DIRECT ? mx : nullptr;
    double* dy = mode != TK_HOST_IO_STAGED ? my : nullptr;
    if (!mx || !my) {
        // pageable buffers: plain stream-ordered copies (graphs take page-locked memory only)
        TK_CUDA(cudaMemcpyAsync(plan->hx.p, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        st = tk_heff2_apply_prec(plan, plan->hx.p, plan->hy.p, s, plan->precision);
        if (st != TK_OK) return st;
        TK_CUDA(cudaMemcpyAsync(y, plan->hy.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        return finish_host_call(plan, s);
    }
    // page-locked buffers: the whole call (copies, kernels, error-word
    // read-back) as one CUDA graph launch, re-instantiated when the buffers
    // or settings change
    const int key = (((mode * 4 + plan->precision) * 4 + plan->schedule) * 16 + plan->psi_pieces) * 4 + (dx ? 2 : 0) +
                    (dy ? 1 : 0);
    if (!plan->host_exec || plan->host_gx != x || plan->host_gy != y || plan->host_gmx != mx ||
        plan->host_gmy != my || plan->host_gkey != key) {
        if (plan->host_exec) {
            cudaGraphExecDestroy(plan->host_exec);
            plan->host_exec = nullptr;
        }
        int64_t x_cut[kTcPsiPieces + 1];
        int32_t n1_cut[kTcPsiPieces + 1];
        const bool pieces = !dx && plan->precision == TK_PREC_BF16X3 &&
                            tc_psi_pieces(*plan->tc, plan->psi_pieces, x_cut, n1_cut);
        TK_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        tk_status cst = TK_OK;
        cudaError_t ce = cudaSuccess;
        if (pieces) {
            cst = enqueue_split_psi_pieces(plan, x, dy ? dy : plan->hy.p, plan->psi_pieces, x_cut, n1_cut, s);
        } else {
            if (!dx) ce = cudaMemcpyAsync(plan->hx.p, x, sizeof(double) * n, cudaMemcpyHostToDevice, s);
            if (ce == cudaSuccess)
                cst = tk_heff2_apply_prec(plan, dx ? dx : plan->hx.p, dy ? dy : plan->hy.p, s, plan->precision);
        }
        if (ce == cudaSuccess && cst == TK_OK && !dy)
            ce = cudaMemcpyAsync(y, plan->hy.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
        if (ce == cudaSuccess && cst == TK_OK && plan->precision == TK_PREC_BF16X3)
            ce = cudaMemcpyAsync(plan->pin_err, tc_error_word(*plan->tc), sizeof(int), cudaMemcpyDeviceToHost, s);
        cudaGraph_t graph = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(s, &graph);
        if (cst != TK_OK) {
            if (graph) cudaGraphDestroy(graph);
            return cst;
        }
        if (ce == cudaSuccess) ce = ee;
        if (ce == cudaSuccess) ce = cudaGraphInstantiate(&plan->host_exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (ce != cudaSuccess) {
            plan->host_exec = nullptr;
            return cuda_fail("tk_heff2_apply_host_flat: graph capture", ce);
        }
        plan->host_gx = x;
        plan->host_gy = y;
        plan->host_gmx = mx;
        plan->host_gmy = my;
        plan->host_gkey = key;
    }
    TK_CUDA(cudaGraphLaunch(plan->host_exec, s));
    TK_CUDA(cudaStreamSynchronize(s));
    if (plan->precision == TK_PREC_BF16X3 && *plan->pin_err != 0) return tc_check_error(*plan->tc, s);
    return TK_OK;
}

tk_status tk_heff2_apply_host(tk_heff2_plan* plan, const double* x, double* y) {
    if (!plan || !x || !y) {
        set_error("tk_heff2_apply_host: null argument");
        return TK_ERR_INVALID_ARG;
    }
    DeviceGuard g(plan->device);
    tk_status st = ensure_host_staging(plan);
    if (st != TK_OK) return st;
    tk_heff2_dense_to_flat(plan, x, plan->pin_x);
    const int64_t n = plan->host.total;
    cudaStream_t s = plan->stream;
    if (n > 0) {
        TK_CUDA(cudaMemcpyAsync(plan->hx.p, plan->pin_x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        st = tk_heff2_apply_prec(plan, plan->hx.p, plan->hy.p, s, plan->precision);
        if (st != TK_OK) return st;
        TK_CUDA(cudaMemcpyAsync(plan->pin_y, plan->hy.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        if ((st = finish_host_call(plan, s)) != TK_OK) return st;
    }
    return tk_heff2_flat_to_dense(plan, plan->pin_y, y);
}

}  // extern "C"

extern "C" tk_status tk_check_split_conversions(tk_ctx* ctx, const double* x_dev, int64_t n, uint64_t* mismatches) {
    if (!ctx || !mismatches || (n > 0 && !x_dev) || n < 0) {
        set_error("tk_check_split_conversions: invalid argument");
        return TK_ERR_INVALID_ARG;
    }
    DeviceGuard g(ctx->device);
    if (!g.ok) {
        set_error("tk_check_split_conversions: cudaSetDevice failed");
        return TK_ERR_CUDA;
    }
    unsigned long long* d = nullptr;
    TK_CUDA(cudaMalloc(&d, sizeof(unsigned long long)));
    unsigned long long h = 0;
    cudaError_t e = cudaMemset(d, 0, sizeof(h));
    if (e == cudaSuccess) e = tc_conversion_check(x_dev, n, d, 0);
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail("tk_check_split_conversions", e);
    *mismatches = h;
    return TK_OK;
}

extern "C" tk_status tk_heff2_profile(tk_heff2_plan* plan, const double* x_dev, double* y_dev, void* stream,
                                      int32_t reps, float* ms, double* flops, double* bytes) {
    if (!plan || !x_dev || !y_dev || !ms || reps < 1) {
        set_error("tk_heff2_profile: invalid argument");
        return TK_ERR_INVALID_ARG;
    }
    DeviceGuard g(plan->device);
    cudaStream_t s = (cudaStream_t)stream;
    tk_heff2_plan* p = plan;
    const Heff2Tables& H = p->host;
    if (flops) {
        flops[0] = H.g1.flops;
        flops[1] = H.comb_flops;
        flops[2] = H.g3.flops;
    }
    if (bytes) {
        if (p->precision == TK_PREC_BF16X3) {
            const TcTables& C = H.tc;
            const double b16 = 2.0 * 2.0 * kTcBK;  // hi + lo bf16 per operand row element x 64
            // T1 reads of the combine kernel and of the fused stage 3, each at
            // most all of T1 (a T1 element read by several terms counts once)
            double comb_reads = 0.0;
            for (const TcCombJob& j : C.jobs) comb_reads += (double)j.rows * j.cols * (j.term_end - j.term_begin);
            const double t1_comb = 4.0 * std::min<double>((double)C.t1_total, comb_reads);
            const double t1_fused = 4.0 * std::min<double>((double)C.t1_total, C.fill_term_elems);
            bytes[0] = 8.0 * H.total + b16 * (double)C.lq_rows + 4.0 * C.t1_total;
            bytes[1] = C.jobs.empty() ? 0.0 : t1_comb + b16 * (double)C.t2q_rows;
            bytes[2] = b16 * (double)C.t2q_rows + t1_fused + b16 * (double)C.rq_rows + 8.0 * H.total;
        } else if (p->schedule == TK_SCHED_STACKED) {
            f64stack_bytes(*p->f64s, bytes);
            bytes[0] += 8.0 * H.total;
            bytes[2] += 8.0 * H.total;
        } else {
            bytes[0] = 8.0 * ((double)H.lbuf.size() + H.total + H.t1_total);
            bytes[1] = 8.0 * ((double)H.t1_total + H.t2_total);
            bytes[2] = 8.0 * ((double)H.t2_total + H.rbuf.size() + H.total);
        }
    }
    cudaEvent_t ev[4];
    for (int i = 0; i < 4; ++i) TK_CUDA(cudaEventCreate(&ev[i]));
    struct EvFree {
        cudaEvent_t* e;
        ~EvFree() {
            for (int i = 0; i < 4; ++i) cudaEventDestroy(e[i]);
        }
    } evf{ev};
    double acc[3] = {0.0, 0.0, 0.0};
    for (int r = 0; r < reps; ++r) {
        TK_CUDA(cudaEventRecord(ev[0], s));
        for (int stage = 0; stage < 3; ++stage) {
            if (p->precision == TK_PREC_BF16X3) {
                std::string err;
                cudaError_t e = tc_apply_stage(*p->tc, p->host, p->jobs.p, p->n_jobs, p->terms.p, x_dev, y_dev, s,
                                               stage, err);
                if (e != cudaSuccess) return cuda_fail(err.c_str(), e);
            } else if (p->schedule == TK_SCHED_STACKED) {
                TK_CUDA(f64stack_stage(*p->f64s, x_dev, y_dev, s, stage));
            } else if (stage == 0) {
                if (p->schedule == TK_SCHED_PER_BLOCK)
                    TK_CUDA(launch_per_block(p->g1, p->lbuf.p, x_dev, p->t1.p, s));
                else
                    TK_CUDA(launch_gemm_f64(p->g1.tiles.p, p->g1.n_tiles, p->g1.tasks.p, p->g1.segs.p, p->lbuf.p,
                                            x_dev, p->t1.p, s));
            } else if (stage == 1) {
                TK_CUDA(launch_combine_f64(p->jobs.p, p->n_jobs, p->terms.p, p->t1.p, p->t2.p, s));
            } else {
                if (p->schedule == TK_SCHED_PER_BLOCK)
                    TK_CUDA(launch_per_block(p->g3, p->t2.p, p->rbuf.p, y_dev, s));
                else
                    TK_CUDA(launch_gemm_f64(p->g3.tiles.p, p->g3.n_tiles, p->g3.tasks.p, p->g3.segs.p, p->t2.p,
                                            p->rbuf.p, y_dev, s));
            }
            TK_CUDA(cudaEventRecord(ev[stage + 1], s));
        }
        TK_CUDA(cudaEventSynchronize(ev[3]));
        for (int stage = 0; stage < 3; ++stage) {
            float t = 0.f;
            TK_CUDA(cudaEventElapsedTime(&t, ev[stage], ev[stage + 1]));
            acc[stage] += t;
        }
    }
    for (int stage = 0; stage < 3; ++stage) ms[stage] = (float)(acc[stage] / reps);
    return TK_OK;
}

namespace {

// Sector-size histogram class of a plan: quantum-number kind, physical and
// MPO dimensions, and for both bonds the log2 buckets of the sector count,
// the largest sector and the total dimension (the bonds of one sweep's
// middle share a class, so the timing is paid once per class).
std::vector<int64_t> histogram_class(const tk_heff2_plan* p) {
    const Heff2Tables& H = p->host;
    std::vector<int64_t> key = {H.kind, H.d_i, H.d_j, H.nwl, H.nwr};
    if (!H.tcsrc) return key;
    for (const QIndex* q : {&H.tcsrc->QA, &H.tcsrc->QB}) {
        int64_t mx = 0;
        for (int64_t d : q->dim) mx = std::max(mx, d);
        auto lg = [](double v) { return (int64_t)std::floor(std::log2(std::max(v, 1.0))); };
        key.push_back(lg((double)q->n()));
        key.push_back(lg((double)mx));
        key.push_back(lg((double)q->total));
    }
    return key;
}

std::mutex g_tune_mutex;
std::map<std::vector<int64_t>, TcOptions> g_tune_cache;

}  // namespace

extern "C" tk_status tk_heff2_autotune(tk_heff2_plan* plan, int32_t reps, int32_t use_cache,
                                       tk_autotune_result* out) {
    if (!plan || !out || reps < 1) {
        set_error("tk_heff2_autotune: invalid argument");
        return TK_ERR_INVALID_ARG;
    }
    std::memset(out, 0, sizeof(*out));
    if (plan->is_complex || plan->precision != TK_PREC_BF16X3 || !plan->tc) {
        set_error("tk_heff2_autotune: tunes split-precision plans only");
        return TK_ERR_UNSUPPORTED;
    }
    DeviceGuard g(plan->device);
    const std::vector<int64_t> key = histogram_class(plan);
    if (use_cache) {
        TcOptions hit;
        bool found = false;
        {
            std::lock_guard<std::mutex> lock(g_tune_mutex);
            auto it = g_tune_cache.find(key);
            if (it != g_tune_cache.end()) {
                hit = it->second;
                found = true;
            }
        }
        if (found) {
            tk_status st = TK_OK;
            if (hit.tall_max_mtiles != plan->host.tcopt.tall_max_mtiles ||
                hit.fuse_max_ntiles != plan->host.tcopt.fuse_max_ntiles ||
                hit.combine_warps != plan->host.tcopt.combine_warps ||
                hit.stage1_persistent != plan->host.tcopt.stage1_persistent ||
                hit.stage1_narrow != plan->host.tcopt.stage1_narrow)
                st = apply_tc_options(plan, hit);
            if (st != TK_OK) return st;
            out->chosen = {hit.tall_max_mtiles, hit.fuse_max_ntiles, hit.combine_warps, hit.stage1_persistent,
                           hit.stage1_narrow};
            out->from_cache = 1;
            return TK_OK;
        }
    }
    const int64_t n = plan->host.total;
    if (n == 0) return TK_OK;
    tk_status st = ensure_host_staging(plan);
    if (st != TK_OK) return st;
    cudaStream_t s = plan->stream;
    TK_CUDA(launch_fill_start_vector(plan->hx.p, n, s));
    // candidate schedules (each stage-1 form with 64- and 32-wide K chunks); a
    // candidate whose tables and launch forms come out the same as an earlier
    // one's is not timed again.  The combine as persistent warps or one
    // warp per job and the fused stage 3 stay settable (tk_heff2_set_tc_options)
    // but are not timed here: 1.3-3.5x slower than the default on the Hubbard
    // D=2048 bond, and every candidate costs a table rebuild inside a sweep
    const TcOptions cand[] = {{3, 0, 0, 0, 0}, {3, 0, 0, 0, 1}, {3, 0, 3, 0, 0}, {3, 0, 3, 0, 1},
                              {3, 0, 0, 1, 0}, {1 << 30, 0, 0, 0, 0}, {1, 0, 0, 0, 0}};
    std::vector<std::vector<size_t>> shapes;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    TK_CUDA(cudaEventCreate(&e0));
    TK_CUDA(cudaEventCreate(&e1));
    struct EvFree {
        cudaEvent_t a, b;
        ~EvFree() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } evf{e0, e1};
    TcOptions best = plan->host.tcopt;
    float best_ms = 1e30f;
    for (const TcOptions& c : cand) {
        if ((st = apply_tc_options(plan, c)) != TK_OK) return st;
        const TcTables& C = plan->host.tc;
        std::vector<size_t> shape = {C.tiles1.size(), C.tiles1x.size(), C.split.size(), C.tiles3.size(),
                                     C.tiles3f.size(), C.jobs.size(), C.jobs.empty() ? 0u : (size_t)c.combine_warps,
                                     C.tiles1.empty() ? 0u : (size_t)c.stage1_persistent,
                                     C.tiles1.empty() || c.stage1_persistent ? 0u : (size_t)c.stage1_narrow};
        if (std::find(shapes.begin(), shapes.end(), shape) != shapes.end()) continue;
        shapes.push_back(shape);
        for (int w = 0; w < 2; ++w)
            if ((st = tk_heff2_apply_prec(plan, plan->hx.p, plan->hy.p, s, TK_PREC_BF16X3)) != TK_OK) return st;
        TK_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < reps; ++r)
            if ((st = tk_heff2_apply_prec(plan, plan->hx.p, plan->hy.p, s, TK_PREC_BF16X3)) != TK_OK) return st;
        TK_CUDA(cudaEventRecord(e1, s));
        TK_CUDA(cudaEventSynchronize(e1));
        if ((st = tc_check_error(*plan->tc, s)) != TK_OK) return st;
        float ms = 0.f;
        TK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        ms /= (float)reps;
        if (out->n_candidates < 8) {
            out->candidates[out->n_candidates] = {c.tall_max_mtiles, c.fuse_max_ntiles, c.combine_warps,
                                                  c.stage1_persistent, c.stage1_narrow};
            out->candidate_ms[out->n_candidates] = ms;
            ++out->n_candidates;
        }
        if (ms < best_ms) {
            best_ms = ms;
            best = c;
        }
    }
    if ((st = apply_tc_options(plan, best)) != TK_OK) return st;
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tune_cache[key] = best;
    }
    out->chosen = {best.tall_max_mtiles, best.fuse_max_ntiles, best.combine_warps, best.stage1_persistent,
                   best.stage1_narrow};
    out->chosen_ms = best_ms;
    return TK_OK;
}
