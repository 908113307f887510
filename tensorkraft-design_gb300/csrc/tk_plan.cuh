// tk_plan.cuh -- device-side state of a two-site H_eff plan.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <string>
#include <vector>

#include "tc_gemm.cuh"
#include "tk_internal.hpp"

namespace tk {

// Device allocations of a plan.  With a countdown armed by
// tk_debug_fail_device_alloc, the countdown-th allocation fails as if the
// device were out of memory (test hook for the TK_ERR_OOM paths).
extern std::atomic<int> g_fail_device_alloc;
inline cudaError_t dev_malloc(void** p, size_t bytes) {
    int c = g_fail_device_alloc.load(std::memory_order_relaxed);
    while (c > 0 && !g_fail_device_alloc.compare_exchange_weak(c, c - 1)) {
    }
    if (c == 1) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { reset(); }
    void reset() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t alloc(size_t count) {
        reset();
        n = count;
        if (count == 0) return cudaSuccess;
        return dev_malloc((void**)&p, sizeof(T) * count);
    }
    cudaError_t upload(const std::vector<T>& v) {
        cudaError_t e = alloc(v.size());
        if (e != cudaSuccess || v.empty()) return e;
        return cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
    }
};

struct DevGemm {
    DevBuf<GemmTask> tasks;
    DevBuf<GemmSeg> segs;
    DevBuf<GemmTile> tiles;
    int n_tiles = 0;
    // the same tiles grouped by task, for the one-launch-per-block schedule
    DevBuf<GemmTile> tiles_by_task;
    std::vector<int> task_tile_begin;  // n_tasks + 1 offsets into tiles_by_task
    cudaError_t upload(const GemmTable& g) {
        cudaError_t e;
        if ((e = tasks.upload(g.tasks)) != cudaSuccess) return e;
        if ((e = segs.upload(g.segs)) != cudaSuccess) return e;
        if ((e = tiles.upload(g.tiles)) != cudaSuccess) return e;
        n_tiles = (int)g.tiles.size();
        std::vector<GemmTile> by(g.tiles);
        std::stable_sort(by.begin(), by.end(), [](const GemmTile& a, const GemmTile& b) { return a.task < b.task; });
        task_tile_begin.assign(g.tasks.size() + 1, 0);
        for (const GemmTile& t : by) task_tile_begin[t.task + 1]++;
        for (size_t i = 1; i < task_tile_begin.size(); ++i) task_tile_begin[i] += task_tile_begin[i - 1];
        return tiles_by_task.upload(by);
    }
};


struct LanczosGraph;
struct LanczosGraphDeleter {
    void operator()(LanczosGraph* g) const;
};

// The stacked FP64 schedule's device operands (stack_f64.cu), built from
// Heff2Tables::f64st on the first TK_SCHED_STACKED request.
struct F64Stack;
struct F64StackDeleter {
    void operator()(F64Stack* p) const;
};
tk_status f64stack_create(const TcTables& C, std::unique_ptr<F64Stack, F64StackDeleter>& out, std::string& err);
// stage 0: T1 = L stacks * psi; 1: the W_i W_j combine into T2; 2: y = T2 * R stacks
cudaError_t f64stack_stage(F64Stack& p, const double* x, double* y, cudaStream_t s, int stage);
cudaError_t f64stack_apply(F64Stack& p, const double* x, double* y, cudaStream_t s);
// The complex matvec (planar vectors) of a stack built from complex environments.
cudaError_t f64stack_apply_complex(F64Stack& p, const double* xr, const double* xi, double* yr, double* yi,
                                   cudaStream_t s);
int f64stack_launches(const F64Stack& p);
// Bytes per stage a stacked matvec must move, without the psi and y vectors.
void f64stack_bytes(const F64Stack& p, double out[3]);

}  // namespace tk

struct tk_heff2_plan {
    int device = 0;
    int precision = TK_PREC_FP64;
    int schedule = TK_SCHED_GROUPED;
    tk::Heff2Tables host;
    tk::DevBuf<double> lbuf, rbuf, t1, t2;
    // complex environments (planar): imaginary parts of the slabs and intermediates
    bool is_complex = false;
    tk::DevBuf<double> lbuf_im, rbuf_im, t1_im, t2_im;
    tk::DevGemm g1, g3;
    bool grouped_ready = false;  // lbuf, rbuf, t1, t2, g1, g3, jobs, terms uploaded (tk::ensure_grouped)
    tk::DevBuf<tk::CombJob> jobs;
    tk::DevBuf<tk::CombTerm> terms;
    int n_jobs = 0;
    // host-call staging (allocated on first host call)
    tk::DevBuf<double> hx, hy;
    double* pin_x = nullptr;
    double* pin_y = nullptr;
    int* pin_err = nullptr;   // tensor-core error word, read back with the result
    int host_io = TK_HOST_IO_AUTO;
    // CUDA graph of the last host-buffer matvec (copies, kernels, error-word
    // read-back), reused while the buffers and the plan settings repeat
    cudaGraphExec_t host_exec = nullptr;
    cudaStream_t copy_stream = nullptr;  // the psi copy of a host-buffer matvec, in pieces
    cudaEvent_t ev_fork = nullptr, ev_piece[tk::kTcPsiPieces] = {};
    int psi_pieces = 2;  // host-buffer psi copy in this many pieces (tk_heff2_set_psi_pieces)
    const void* host_gx = nullptr;
    void* host_gy = nullptr;
    // device addresses of x and y's page-locked mappings when the graph was made
    // (a buffer freed and re-registered at the same host address can map elsewhere)
    const void* host_gmx = nullptr;
    const void* host_gmy = nullptr;
    int host_gkey = -1;
    cudaStream_t stream = nullptr;
    // host cancel flag (tk_heff2_set_cancel_flag), polled between eigensolver iterations
    const int32_t* cancel = nullptr;
    // split-precision operands and state (tensor-core path)
    std::unique_ptr<tk::TcPlan, tk::TcPlanDeleter> tc;
    // stacked FP64 operands (TK_SCHED_STACKED)
    std::unique_ptr<tk::F64Stack, tk::F64StackDeleter> f64s;
    // Lanczos workspace (allocated on first use)
    tk::DevBuf<double> lz_basis, lz_w, lz_scal, lz_part, lz_vec;
    // FP64 search space of the Davidson / refinement solver (allocated on first use)
    tk::DevBuf<double> sub_v, sub_hv, sub_sc, sub_part;
    int sub_cap = 0;
    // Krylov-exponential workspace (allocated on first use)
    tk::DevBuf<double> ex_basis, ex_w, ex_x2, ex_scal, ex_part;
    int ex_cap_m = 0;
    int64_t ex_cap_n = 0;
    int lz_cap_k = 0;
    std::unique_ptr<tk::LanczosGraph, tk::LanczosGraphDeleter> lz_graph;
    ~tk_heff2_plan() {
        if (pin_x) cudaFreeHost(pin_x);
        if (pin_y) cudaFreeHost(pin_y);
        if (pin_err) cudaFreeHost(pin_err);
        if (host_exec) cudaGraphExecDestroy(host_exec);
        if (ev_fork) cudaEventDestroy(ev_fork);
        for (cudaEvent_t e : ev_piece)
            if (e) cudaEventDestroy(e);
        if (copy_stream) cudaStreamDestroy(copy_stream);
        if (stream) cudaStreamDestroy(stream);
    }
};

// Dispatches one matvec in the requested precision (stream-ordered).
extern "C" tk_status tk_heff2_apply_prec(tk_heff2_plan* p, const double* x, double* y, cudaStream_t s, int precision);
// The complex FP64 matvec of a complex plan on planar vectors (stream-ordered).
extern "C" tk_status tk_heff2_apply_complex_s(tk_heff2_plan* p, const double* xr, const double* xi, double* yr,
                                              double* yi, cudaStream_t s);

namespace tk {
tk_status cuda_fail(const char* op, cudaError_t e);
// Uploads the grouped / per-block FP64 schedules' device state once.
tk_status ensure_grouped(tk_heff2_plan* p);
// True once the plan's cancel flag (if any) reads non-zero: the solver waits
// for its stream, so that none of its work is left in flight, records the
// message and returns TK_ERR_CANCELLED.
bool plan_cancelled(tk_heff2_plan* p, cudaStream_t s, const char* where);
// Plan creation behind tk_heff2_plan_create / tk_heff2_plan_create_dev: with
// l_blocks / r_blocks (host copies of canonical block-layout environments) the
// environments' `data` pointers are not read.  `stacked`: build the stacked
// FP64 operands and make TK_SCHED_STACKED the plan's schedule; without it the
// caller sets a schedule (tk_heff2_set_schedule) before the plan is used.
tk_status plan_create_impl(tk_ctx* ctx, const tk_env* env_l, const tk_env* env_r, const tk_bst* w_i,
                           const tk_bst* w_j, const int32_t* psi_flux, int32_t precision, const double* l_blocks,
                           const double* r_blocks, tk_heff2_plan** out, bool stacked = true);
}
