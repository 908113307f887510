// linalg.cu -- LinAlgBackend::gemm, SparseLinAlgBackend::{block_gemm, spmv}
// on the device, through the same grouped segmented FP64 GEMM kernel as the
// H_eff path.
//
// block_gemm follows tk-linalg/src/device/faer.rs:390-575 and
// tk-linalg/src/tasks.rs:36-81,180-188: a task for every (key_a, key_b) pair
// whose contracted quantum numbers are equal and whose output sector
// satisfies row (+) dual(col) == flux_a (+) flux_b; contributions to the same
// output key are summed (here in registers, one output block per task); the
// output keys are ascending; output legs [a.legs[0], b.legs[1]] with
// directions [a.dirs[0], b.dirs[1]].
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "tk_bsgemm.hpp"
#include "tk_internal.hpp"
#include "tk_plan.cuh"

using namespace tk;

namespace {

struct Guard {
    int prev = -1;
    explicit Guard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        cudaSetDevice(dev);
    }
    ~Guard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

tk_status fail(const char* op, cudaError_t e) {
    set_error(std::string(op) + ": " + cudaGetErrorName(e) + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? TK_ERR_OOM : TK_ERR_CUDA;
}

struct Scratch {
    std::vector<void*> ptrs;
    ~Scratch() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    cudaError_t put(const std::vector<T>& v, T** out) {
        *out = nullptr;
        if (v.empty()) return cudaSuccess;
        cudaError_t e = cudaMalloc((void**)out, sizeof(T) * v.size());
        if (e != cudaSuccess) return e;
        ptrs.push_back(*out);
        return cudaMemcpy(*out, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
    }
    template <class T>
    cudaError_t make(size_t n, T** out) {
        *out = nullptr;
        if (n == 0) return cudaSuccess;
        cudaError_t e = cudaMalloc((void**)out, sizeof(T) * n);
        if (e == cudaSuccess) ptrs.push_back(*out);
        return e;
    }
};

#define CK(op)                                        \
    do {                                              \
        cudaError_t e_ = (op);                        \
        if (e_ != cudaSuccess) return fail(#op, e_);  \
    } while (0)

void tiles_for(GemmTable& g, int task) { bsgemm_tiles_for(g, task); }

}  // namespace

extern "C" {

tk_status tk_gemm_f64(tk_ctx* ctx, double alpha, const tk_mat* a, const tk_mat* b, double beta, tk_mat_mut* c,
                      void* stream) {
    (void)ctx;
    if (!a || !b || !c || !a->data || !b->data || !c->data) {
        set_error("tk_gemm_f64: null argument");
        return TK_ERR_INVALID_ARG;
    }
    if (a->cols != b->rows || c->rows != a->rows || c->cols != b->cols) {
        set_error("tk_gemm_f64: shape mismatch");
        return TK_ERR_INVALID_ARG;
    }
    if (c->rows == 0 || c->cols == 0) return TK_OK;
    const int64_t lim = INT32_MAX;
    if (a->rows > lim || a->cols > lim || b->cols > lim || std::llabs(a->row_stride) > lim ||
        std::llabs(a->col_stride) > lim || std::llabs(b->row_stride) > lim || std::llabs(b->col_stride) > lim ||
        std::llabs(c->row_stride) > lim || std::llabs(c->col_stride) > lim) {
        set_error("tk_gemm_f64: dimensions or strides exceed 32 bits");
        return TK_ERR_UNSUPPORTED;
    }
    GemmTable g;
    GemmTask t{};
    t.M = (int32_t)a->rows;
    t.N = (int32_t)b->cols;
    t.c_off = 0;
    t.c_rs = (int32_t)c->row_stride;
    t.c_cs = (int32_t)c->col_stride;
    t.alpha = alpha;
    t.beta = beta;
    t.seg_begin = 0;
    t.seg_end = a->cols > 0 ? 1 : 0;
    if (a->cols > 0) {
        GemmSeg s{};
        s.a_off = 0; s.a_rs = (int32_t)a->row_stride; s.a_cs = (int32_t)a->col_stride;
        s.b_off = 0; s.b_rs = (int32_t)b->row_stride; s.b_cs = (int32_t)b->col_stride;
        s.K = (int32_t)a->cols;
        g.segs.push_back(s);
    }
    g.tasks.push_back(t);
    tiles_for(g, 0);
    int dev = 0;
    if (ctx) dev = ctx->device;
    Guard gd(dev);
    Scratch sc;
    GemmTask* dt; GemmSeg* ds; GemmTile* dl;
    CK(sc.put(g.tasks, &dt));
    CK(sc.put(g.segs, &ds));
    CK(sc.put(g.tiles, &dl));
    cudaStream_t s = (cudaStream_t)stream;
    CK(launch_gemm_f64(dl, (int)g.tiles.size(), dt, ds, a->data, b->data, c->data, s));
    // The task tables are freed on return; finish the launch first.
    CK(cudaStreamSynchronize(s));
    return TK_OK;
}

// Output header of a block GEMM (legs of A's rows and B's columns, their
// directions, the output flux) and its key / offset arrays; data unallocated.
static tk_status fill_out_header(const tk_bst* a_abi, const tk_bst* b_abi, const Rank2& A, const Rank2& B,
                                 const BlockGemmPlan& P, tk_bst_out* out, bool with_data) {
    out->qn_kind = A.kind;
    out->rank = 2;
    out->legs[0] = a_abi->legs[0];
    out->legs[1] = b_abi->legs[1];
    out->leg_dirs[0] = A.dirs[0];
    out->leg_dirs[1] = B.dirs[1];
    out->flux[0] = P.target.c[0];
    out->flux[1] = P.target.c[1];
    out->n_blocks = (int64_t)P.okeys.size();
    out->total = P.total;
    out->keys = (uint64_t*)std::malloc(sizeof(uint64_t) * std::max<size_t>(P.okeys.size(), 1));
    out->block_offsets = (int64_t*)std::malloc(sizeof(int64_t) * std::max<size_t>(P.ooffs.size(), 1));
    out->data = with_data ? (double*)std::malloc(sizeof(double) * (size_t)std::max<int64_t>(P.total, 1)) : nullptr;
    if (!out->keys || !out->block_offsets || (with_data && !out->data)) {
        tk_bst_free(out);
        set_error("block gemm: host allocation failed");
        return TK_ERR_OOM;
    }
    std::copy(P.okeys.begin(), P.okeys.end(), out->keys);
    std::copy(P.ooffs.begin(), P.ooffs.end(), out->block_offsets);
    return TK_OK;
}

// Grouped-GEMM tables of a block GEMM, packed for one copy.
struct TableBlob {
    size_t tasks = 0, segs = 0, tiles = 0;
};
static TableBlob add_tables(Blob& b, const GemmTable& g) {
    TableBlob t;
    t.tasks = b.add(g.tasks.data(), sizeof(GemmTask) * g.tasks.size());
    t.segs = b.add(g.segs.data(), sizeof(GemmSeg) * g.segs.size());
    t.tiles = b.add(g.tiles.data(), sizeof(GemmTile) * g.tiles.size());
    return t;
}

// Copies `blob` through the context's page-locked staging into its device
// scratch on `s`; *dev receives the scratch base (at least blob.device_size()).
static tk_status stage_blob(tk_ctx* ctx, const Blob& blob, cudaStream_t s, unsigned char** dev) {
    void *d = nullptr, *h = nullptr;
    tk_status st;
    if ((st = ctx_dev_scratch(ctx, blob.device_size(), &d)) != TK_OK) return st;
    if ((st = ctx_host_stage(ctx, std::max<size_t>(blob.size(), 1), &h)) != TK_OK) return st;
    blob.copy_to(h);
    if (!(blob.size() == 0)) CK(cudaMemcpyAsync(d, h, blob.size(), cudaMemcpyHostToDevice, s));
    *dev = static_cast<unsigned char*>(d);
    return TK_OK;
}

tk_status tk_block_gemm_f64(tk_ctx* ctx, const tk_bst* a_abi, const tk_bst* b_abi, tk_bst_out* out) {
    if (!ctx || !a_abi || !b_abi || !out) {
        set_error("tk_block_gemm_f64: null argument");
        return TK_ERR_INVALID_ARG;
    }
    std::memset(out, 0, sizeof(*out));
    std::string err;
    Rank2 A, B;
    if (!rank2_from_abi(*a_abi, A, "A", err) || !rank2_from_abi(*b_abi, B, "B", err)) {
        set_error("tk_block_gemm_f64: " + err);
        return TK_ERR_INVALID_ARG;
    }
    BlockGemmPlan P;
    tk_status st = guard_host("tk_block_gemm_f64", err, [&] { return block_gemm_plan(A, B, P, err); });
    if (st != TK_OK) {
        set_error("tk_block_gemm_f64: " + err);
        return st;
    }
    if ((st = fill_out_header(a_abi, b_abi, A, B, P, out, true)) != TK_OK) return st;
    if (P.total == 0) return TK_OK;
    Guard gd(ctx->device);
    // one host-to-device copy: A, B and the tables; C is written on the device
    // and read back through the same staging buffer
    Blob blob;
    const size_t oa = blob.add(A.data, sizeof(double) * (size_t)A.total);
    const size_t ob = blob.add(B.data, sizeof(double) * (size_t)B.total);
    const TableBlob tb = add_tables(blob, P.g);
    const size_t oc = blob.reserve(sizeof(double) * (size_t)P.total);
    auto run = [&]() -> tk_status {
        void* sp = nullptr;
        tk_status s2;
        if ((s2 = ctx_stream(ctx, &sp)) != TK_OK) return s2;
        cudaStream_t s = (cudaStream_t)sp;
        unsigned char* d = nullptr;
        if ((s2 = ctx_host_stage(ctx, sizeof(double) * (size_t)P.total, &sp)) != TK_OK) return s2;
        if ((s2 = stage_blob(ctx, blob, s, &d)) != TK_OK) return s2;
        CK(launch_gemm_f64((const GemmTile*)(d + tb.tiles), (int)P.g.tiles.size(), (const GemmTask*)(d + tb.tasks),
                           (const GemmSeg*)(d + tb.segs), (const double*)(d + oa), (const double*)(d + ob),
                           (double*)(d + oc), s));
        CK(cudaMemcpyAsync(ctx->host_stage, d + oc, sizeof(double) * (size_t)P.total, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        std::memcpy(out->data, ctx->host_stage, sizeof(double) * (size_t)P.total);
        return TK_OK;
    };
    st = run();
    if (st != TK_OK) tk_bst_free(out);
    return st;
}

tk_status tk_block_gemm_f64_dev(tk_ctx* ctx, const tk_bst* a_abi, const tk_bst* b_abi, tk_bst_out* out,
                                double* c_dev, void* stream) {
    if (!ctx || !a_abi || !b_abi || !out) {
        set_error("tk_block_gemm_f64_dev: null argument");
        return TK_ERR_INVALID_ARG;
    }
    std::memset(out, 0, sizeof(*out));
    std::string err;
    Rank2 A, B;
    if (!rank2_from_abi(*a_abi, A, "A", err) || !rank2_from_abi(*b_abi, B, "B", err)) {
        set_error("tk_block_gemm_f64_dev: " + err);
        return TK_ERR_INVALID_ARG;
    }
    BlockGemmPlan P;
    tk_status st = guard_host("tk_block_gemm_f64_dev", err, [&] { return block_gemm_plan(A, B, P, err); });
    if (st != TK_OK) {
        set_error("tk_block_gemm_f64_dev: " + err);
        return st;
    }
    if ((st = fill_out_header(a_abi, b_abi, A, B, P, out, false)) != TK_OK) return st;
    if (!c_dev || P.total == 0) return TK_OK;
    Guard gd(ctx->device);
    Blob blob;
    const TableBlob tb = add_tables(blob, P.g);
    cudaStream_t s = (cudaStream_t)stream;
    auto run = [&]() -> tk_status {
        unsigned char* d = nullptr;
        tk_status s2 = stage_blob(ctx, blob, s, &d);
        if (s2 != TK_OK) return s2;
        CK(launch_gemm_f64((const GemmTile*)(d + tb.tiles), (int)P.g.tiles.size(), (const GemmTask*)(d + tb.tasks),
                           (const GemmSeg*)(d + tb.segs), A.data, B.data, c_dev, s));
        // the tables live in the context's shared scratch: finish before returning
        CK(cudaStreamSynchronize(s));
        return TK_OK;
    };
    st = run();
    if (st != TK_OK) tk_bst_free(out);
    return st;
}

void tk_bst_free(tk_bst_out* t) {
    if (!t) return;
    std::free(t->keys);
    std::free(t->block_offsets);
    std::free(t->data);
    std::free(t->owned_charges);
    std::free(t->owned_dims);
    t->keys = nullptr;
    t->block_offsets = nullptr;
    t->data = nullptr;
    t->owned_charges = nullptr;
    t->owned_dims = nullptr;
    t->n_blocks = 0;
    t->total = 0;
}

tk_status tk_spmv_f64(tk_ctx* ctx, const tk_bst* a_abi, const double* x, double* y) {
    if (!a_abi || !x || !y) {
        set_error("tk_spmv_f64: null argument");
        return TK_ERR_INVALID_ARG;
    }
    std::string err;
    Rank2 A;
    if (!rank2_from_abi(*a_abi, A, "A", err)) {
        set_error("tk_spmv_f64: " + err);
        return TK_ERR_INVALID_ARG;
    }
    const int64_t rows = A.legs[0].total, cols = A.legs[1].total;
    // One task per row sector (faer.rs:336-388: y zeroed, each block adds
    // its product into its row range); blocks of one row sector are K segments.
    GemmTable g;
    std::map<int, std::vector<int>> by_row;
    for (size_t b = 0; b < A.keys.size(); ++b) by_row[A.rs[b]].push_back((int)b);
    std::vector<char> covered((size_t)A.legs[0].n(), 0);
    for (auto& kv : by_row) {
        int r = kv.first;
        covered[r] = 1;
        GemmTask t{};
        t.M = (int32_t)A.legs[0].dim[r]; t.N = 1;
        t.c_off = A.legs[0].off[r]; t.c_rs = 1; t.c_cs = 1;
        t.alpha = 1.0; t.beta = 0.0;
        t.seg_begin = (int)g.segs.size();
        for (int b : kv.second) {
            int c = A.cs[b];
            GemmSeg s{};
            s.a_off = A.offs[b]; s.a_rs = (int32_t)A.legs[1].dim[c]; s.a_cs = 1;
            s.b_off = A.legs[1].off[c]; s.b_rs = 1; s.b_cs = 1;
            s.K = (int32_t)A.legs[1].dim[c];
            g.segs.push_back(s);
        }
        t.seg_end = (int)g.segs.size();
        g.tasks.push_back(t);
        tiles_for(g, (int)g.tasks.size() - 1);
    }
    // Row sectors without blocks are zero.
    for (int r = 0; r < A.legs[0].n(); ++r) {
        if (covered[r]) continue;
        GemmTask t{};
        t.M = (int32_t)A.legs[0].dim[r]; t.N = 1;
        t.c_off = A.legs[0].off[r]; t.c_rs = 1; t.c_cs = 1;
        t.alpha = 1.0; t.beta = 0.0;
        t.seg_begin = t.seg_end = (int)g.segs.size();
        g.tasks.push_back(t);
        tiles_for(g, (int)g.tasks.size() - 1);
    }
    if (rows == 0) return TK_OK;
    int dev = ctx ? ctx->device : 0;
    Guard gd(dev);
    Scratch sc;
    double *da, *dx, *dy;
    GemmTask* dt; GemmSeg* ds; GemmTile* dl;
    std::vector<double> ha(A.data, A.data + A.total), hx(x, x + cols);
    CK(sc.put(ha, &da));
    CK(sc.put(hx, &dx));
    CK(sc.make((size_t)rows, &dy));
    CK(sc.put(g.tasks, &dt));
    CK(sc.put(g.segs, &ds));
    CK(sc.put(g.tiles, &dl));
    CK(launch_gemm_f64(dl, (int)g.tiles.size(), dt, ds, da, dx, dy, nullptr));
    CK(cudaMemcpy(y, dy, sizeof(double) * (size_t)rows, cudaMemcpyDeviceToHost));
    return TK_OK;
}

}  // extern "C"
