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
#include "tk_internal.hpp"

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

void tiles_for(GemmTable& g, int task) {
    const GemmTask& t = g.tasks[task];
    for (int m0 = 0; m0 < t.M; m0 += kF64TileM)
        for (int n0 = 0; n0 < t.N; n0 += kF64TileN) g.tiles.push_back({task, m0, n0, 0});
}

struct Rank2 {
    int kind = 0;
    QIndex legs[2];
    int8_t dirs[2] = {0, 0};
    Qn flux;
    std::vector<uint64_t> keys;
    std::vector<int64_t> offs;
    std::vector<int> rs, cs;  // sector index per block
    const double* data = nullptr;
    int64_t total = 0;
};

bool rank2_from_abi(const tk_bst& t, Rank2& o, const char* name, std::string& err) {
    if (t.rank != 2 || !t.legs || !qn_kind_valid(t.qn_kind)) {
        err = std::string(name) + ": rank-2 tensor with a known quantum-number kind required";
        return false;
    }
    o.kind = t.qn_kind;
    for (int l = 0; l < 2; ++l) {
        if (!qindex_from_abi(t.qn_kind, t.legs[l], o.legs[l], err)) return false;
        o.dirs[l] = t.leg_dirs ? t.leg_dirs[l] : (int8_t)l;
    }
    if (t.flux)
        for (int k = 0; k < qn_ncomp(t.qn_kind); ++k) o.flux.c[k] = t.flux[k];
    if (t.n_blocks > 0 && (!t.keys || !t.block_offsets || !t.data)) {
        err = std::string(name) + ": null block arrays";
        return false;
    }
    o.data = t.data;
    for (int64_t b = 0; b < t.n_blocks; ++b) {
        Qn q[2];
        key_unpack(t.qn_kind, t.keys[b], 2, q);
        int r = o.legs[0].find(q[0]), c = o.legs[1].find(q[1]);
        if (r < 0 || c < 0) {
            err = std::string(name) + ": block key names a sector missing from its QIndex";
            return false;
        }
        if (b > 0 && t.keys[b - 1] >= t.keys[b]) {
            err = std::string(name) + ": keys not strictly ascending";
            return false;
        }
        o.keys.push_back(t.keys[b]);
        o.offs.push_back(t.block_offsets[b]);
        o.rs.push_back(r);
        o.cs.push_back(c);
        o.total = std::max(o.total, t.block_offsets[b] + o.legs[0].dim[r] * o.legs[1].dim[c]);
    }
    return true;
}

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

tk_status tk_block_gemm_f64(tk_ctx* ctx, const tk_bst* a_abi, const tk_bst* b_abi, tk_bst_out* out) {
    if (!a_abi || !b_abi || !out) {
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
    if (A.kind != B.kind) {
        set_error("tk_block_gemm_f64: quantum-number kinds differ");
        return TK_ERR_INVALID_ARG;
    }
    const int kind = A.kind;
    const Qn target = qn_fuse(kind, A.flux, B.flux);
    // Phase 1 (faer.rs:406-430): task generation per compatible pair.
    std::map<uint64_t, std::vector<std::pair<int, int>>> by_out;
    for (size_t i = 0; i < A.keys.size(); ++i)
        for (size_t j = 0; j < B.keys.size(); ++j) {
            const Qn& qa_col = A.legs[1].q[A.cs[i]];
            const Qn& qb_row = B.legs[0].q[B.rs[j]];
            if (qa_col != qb_row) continue;
            Qn out_q[2] = {A.legs[0].q[A.rs[i]], B.legs[1].q[B.cs[j]]};
            if (qn_fuse(kind, out_q[0], qn_dual(kind, out_q[1])) != target) continue;
            if (A.legs[1].dim[A.cs[i]] != B.legs[0].dim[B.rs[j]]) {
                set_error("tk_block_gemm_f64: contracted sector dimensions differ");
                return TK_ERR_SECTOR_MISMATCH;
            }
            by_out[key_pack(kind, out_q, 2)].push_back({(int)i, (int)j});
        }
    // Output blocks in ascending key order (faer.rs:560-574).
    GemmTable g;
    std::vector<uint64_t> okeys;
    std::vector<int64_t> ooffs;
    int64_t total = 0;
    for (auto& kv : by_out) {
        const auto& pairs = kv.second;
        int i0 = pairs[0].first, j0 = pairs[0].second;
        int64_t M = A.legs[0].dim[A.rs[i0]], N = B.legs[1].dim[B.cs[j0]];
        GemmTask t{};
        t.M = (int32_t)M; t.N = (int32_t)N;
        t.c_off = total; t.c_rs = (int32_t)N; t.c_cs = 1;
        t.alpha = 1.0; t.beta = 0.0;
        t.seg_begin = (int)g.segs.size();
        for (auto& pr : pairs) {
            int64_t K = A.legs[1].dim[A.cs[pr.first]];
            GemmSeg s{};
            s.a_off = A.offs[pr.first]; s.a_rs = (int32_t)K; s.a_cs = 1;
            s.b_off = B.offs[pr.second]; s.b_rs = (int32_t)N; s.b_cs = 1;
            s.K = (int32_t)K;
            g.segs.push_back(s);
        }
        t.seg_end = (int)g.segs.size();
        g.tasks.push_back(t);
        tiles_for(g, (int)g.tasks.size() - 1);
        okeys.push_back(kv.first);
        ooffs.push_back(total);
        total += M * N;
    }
    // Fill the output header.
    out->qn_kind = kind;
    out->rank = 2;
    out->legs[0] = a_abi->legs[0];
    out->legs[1] = b_abi->legs[1];
    out->leg_dirs[0] = A.dirs[0];
    out->leg_dirs[1] = B.dirs[1];
    out->flux[0] = target.c[0];
    out->flux[1] = target.c[1];
    out->n_blocks = (int64_t)okeys.size();
    out->total = total;
    out->keys = (uint64_t*)std::malloc(sizeof(uint64_t) * std::max<size_t>(okeys.size(), 1));
    out->block_offsets = (int64_t*)std::malloc(sizeof(int64_t) * std::max<size_t>(ooffs.size(), 1));
    out->data = (double*)std::malloc(sizeof(double) * (size_t)std::max<int64_t>(total, 1));
    if (!out->keys || !out->block_offsets || !out->data) {
        tk_bst_free(out);
        set_error("tk_block_gemm_f64: host allocation failed");
        return TK_ERR_OOM;
    }
    std::copy(okeys.begin(), okeys.end(), out->keys);
    std::copy(ooffs.begin(), ooffs.end(), out->block_offsets);
    if (total == 0) return TK_OK;
    int dev = ctx ? ctx->device : 0;
    Guard gd(dev);
    Scratch sc;
    double *da, *db, *dc;
    GemmTask* dt; GemmSeg* ds; GemmTile* dl;
    std::vector<double> ha(A.data, A.data + A.total), hb(B.data, B.data + B.total);
    tk_status st = TK_OK;
    auto run = [&]() -> tk_status {
        CK(sc.put(ha, &da));
        CK(sc.put(hb, &db));
        CK(sc.make((size_t)total, &dc));
        CK(sc.put(g.tasks, &dt));
        CK(sc.put(g.segs, &ds));
        CK(sc.put(g.tiles, &dl));
        CK(launch_gemm_f64(dl, (int)g.tiles.size(), dt, ds, da, db, dc, nullptr));
        CK(cudaMemcpy(out->data, dc, sizeof(double) * (size_t)total, cudaMemcpyDeviceToHost));
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
    t->keys = nullptr;
    t->block_offsets = nullptr;
    t->data = nullptr;
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
