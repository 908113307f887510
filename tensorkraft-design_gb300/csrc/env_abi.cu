// env_abi.cu -- C ABI of the block-sparse environment operations: canonical
// layout, H_eff plans over device environments, environment growth by one
// site and the two-site start vector (tables in env.cpp).
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "kernels.cuh"
#include "tk_env.hpp"
#include "tk_plan.cuh"

static_assert(tk::kEnvTileM == tk::kF64TileM && tk::kEnvTileN == tk::kF64TileN,
              "environment tables are cut for the grouped FP64 GEMM tile");

using namespace tk;

namespace {

struct Guard {
    int prev = -1;
    bool ok = false;
    explicit Guard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        ok = (cudaSetDevice(dev) == cudaSuccess);
    }
    ~Guard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

// Stream-ordered scratch: allocated from the device's memory pool on the
// call's stream and released on it, so nothing waits on the host.
struct Scratch {
    cudaStream_t s;
    std::vector<void*> ptrs;
    explicit Scratch(cudaStream_t st) : s(st) {}
    ~Scratch() {
        for (void* p : ptrs) cudaFreeAsync(p, s);
    }
    template <class T>
    cudaError_t upload(const std::vector<T>& v, T** out) {
        *out = nullptr;
        if (v.empty()) return cudaSuccess;
        cudaError_t e = alloc(v.size() * sizeof(T), (void**)out);
        if (e != cudaSuccess) return e;
        // pageable source: staged before the call returns
        return cudaMemcpyAsync(*out, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
    }
    cudaError_t alloc(size_t bytes, void** out) {
        cudaError_t e = cudaMallocAsync(out, std::max<size_t>(bytes, 16), s);
        if (e == cudaSuccess) ptrs.push_back(*out);
        return e;
    }
};

tk_status launch_table(Scratch& sc, const GemmTable& g, const double* A, const double* B, double* C) {
    GemmTask* t = nullptr;
    GemmSeg* sg = nullptr;
    GemmTile* tl = nullptr;
    cudaError_t e;
    if ((e = sc.upload(g.tasks, &t)) != cudaSuccess) return cuda_fail("upload tables", e);
    if ((e = sc.upload(g.segs, &sg)) != cudaSuccess) return cuda_fail("upload tables", e);
    if ((e = sc.upload(g.tiles, &tl)) != cudaSuccess) return cuda_fail("upload tables", e);
    if ((e = launch_gemm_f64(tl, (int)g.tiles.size(), t, sg, A, B, C, sc.s)) != cudaSuccess)
        return cuda_fail("grouped gemm", e);
    return TK_OK;
}

// A GEMM table uploaded to stream-ordered scratch.
struct DevTable {
    GemmTask* t = nullptr;
    GemmSeg* sg = nullptr;
    GemmTile* tl = nullptr;
    int n = 0;
    tk_status upload(Scratch& sc, const GemmTable& g) {
        cudaError_t e;
        if ((e = sc.upload(g.tasks, &t)) != cudaSuccess || (e = sc.upload(g.segs, &sg)) != cudaSuccess ||
            (e = sc.upload(g.tiles, &tl)) != cudaSuccess)
            return cuda_fail("upload tables", e);
        n = (int)g.tiles.size();
        return TK_OK;
    }
};

bool env_legs(int kind, const tk_env& e, QIndex& bra, QIndex& mpo, QIndex& ket, std::string& err) {
    return qindex_from_abi(kind, e.bra, bra, err) && qindex_from_abi(kind, e.mpo, mpo, err) &&
           qindex_from_abi(kind, e.ket, ket, err);
}

// env_im / a_im / out_im non-null: complex (planar) environment growth.
tk_status grow(const char* name, bool left, tk_ctx* ctx, const tk_env* env, const tk_bst* a, const tk_bst* w,
               double* out, void* stream, const double* env_im = nullptr, const double* a_im = nullptr,
               double* out_im = nullptr) {
    const bool cplx = env_im || a_im || out_im;
    if (cplx && !(env_im && a_im && out_im)) {
        set_error(std::string(name) + ": complex growth needs every imaginary part");
        return TK_ERR_INVALID_ARG;
    }
    if (!ctx || !env || !a || !w || !out) {
        set_error(std::string(name) + ": null argument");
        return TK_ERR_INVALID_ARG;
    }
    std::string err;
    Bst3 A;
    Bst4 W;
    QIndex eb, em, ek;
    if (!bst3_from_abi(*a, A, "MPS site", err) || !bst4_from_abi(*w, W, "MPO site", err) ||
        !env_legs(A.kind, *env, eb, em, ek, err)) {
        set_error(std::string(name) + ": " + err);
        return TK_ERR_INVALID_ARG;
    }
    if (W.kind != A.kind) {
        set_error(std::string(name) + ": MPS and MPO quantum-number kinds differ");
        return TK_ERR_INVALID_ARG;
    }
    if (!env->data) {
        set_error(std::string(name) + ": null environment data");
        return TK_ERR_INVALID_ARG;
    }
    GrowTables G;
    tk_status st = build_grow_tables(left, eb, em, ek, A, W, G, err);
    if (st != TK_OK) {
        set_error(std::string(name) + ": " + err);
        return st;
    }
    Guard g(ctx->device);
    if (!g.ok) {
        set_error(std::string(name) + ": cudaSetDevice failed");
        return TK_ERR_CUDA;
    }
    cudaStream_t s = (cudaStream_t)stream;
    Scratch sc(s);
    cudaError_t e;
    const size_t parts = cplx ? 2 : 1;
    double *t1 = nullptr, *t2 = nullptr;
    if ((e = sc.alloc(sizeof(double) * parts * (size_t)G.t1_total, (void**)&t1)) != cudaSuccess)
        return cuda_fail("scratch", e);
    if ((e = sc.alloc(sizeof(double) * parts * (size_t)G.t2_total, (void**)&t2)) != cudaSuccess)
        return cuda_fail("scratch", e);
    if ((e = cudaMemsetAsync(out, 0, sizeof(double) * (size_t)G.out_total, s)) != cudaSuccess)
        return cuda_fail("cudaMemsetAsync", e);
    if (cplx && (e = cudaMemsetAsync(out_im, 0, sizeof(double) * (size_t)G.out_total, s)) != cudaSuccess)
        return cuda_fail("cudaMemsetAsync", e);
    CombJob* jobs = nullptr;
    CombTerm* terms = nullptr;
    if ((e = sc.upload(G.jobs, &jobs)) != cudaSuccess) return cuda_fail("upload tables", e);
    if ((e = sc.upload(G.terms, &terms)) != cudaSuccess) return cuda_fail("upload tables", e);
    if (!cplx) {
        if (left)
            st = launch_table(sc, G.g1, env->data, A.data, t1);
        else
            st = launch_table(sc, G.g1, A.data, env->data, t1);
        if (st != TK_OK) return st;
        if ((e = launch_combine_f64(jobs, (int)G.jobs.size(), terms, t1, t2, s)) != cudaSuccess)
            return cuda_fail("combine", e);
        return launch_table(sc, G.g3, A.data, t2, out);
    }
    // complex: stage 1 without conjugation, stage 3 with the bra (site operand) conjugated
    double* t1i = t1 + G.t1_total;
    double* t2i = t2 + G.t2_total;
    DevTable g1, g3;
    if ((st = g1.upload(sc, G.g1)) != TK_OK || (st = g3.upload(sc, G.g3)) != TK_OK) return st;
    if (left)
        e = launch_gemm_c64(g1.tl, g1.n, g1.t, g1.sg, env->data, env_im, A.data, a_im, t1, t1i, false, s);
    else
        e = launch_gemm_c64(g1.tl, g1.n, g1.t, g1.sg, A.data, a_im, env->data, env_im, t1, t1i, false, s);
    if (e != cudaSuccess) return cuda_fail("grouped gemm", e);
    if ((e = launch_combine_f64(jobs, (int)G.jobs.size(), terms, t1, t2, s)) != cudaSuccess ||
        (e = launch_combine_f64(jobs, (int)G.jobs.size(), terms, t1i, t2i, s)) != cudaSuccess)
        return cuda_fail("combine", e);
    if ((e = launch_gemm_c64(g3.tl, g3.n, g3.t, g3.sg, A.data, a_im, t2, t2i, out, out_im, true, s)) != cudaSuccess)
        return cuda_fail("grouped gemm", e);
    return TK_OK;
}

}  // namespace

extern "C" {

tk_status tk_env_layout(int32_t qn_kind, const tk_qindex* bra, const tk_qindex* mpo, const tk_qindex* ket,
                        int64_t* n_blocks, uint64_t* keys, int64_t* block_offsets, int64_t* total) {
    if (!bra || !mpo || !ket || !n_blocks) {
        set_error("tk_env_layout: null argument");
        return TK_ERR_INVALID_ARG;
    }
    if (!qn_kind_valid(qn_kind)) {
        set_error("tk_env_layout: unknown quantum-number kind");
        return TK_ERR_INVALID_ARG;
    }
    std::string err;
    QIndex b, m, k;
    if (!qindex_from_abi(qn_kind, *bra, b, err) || !qindex_from_abi(qn_kind, *mpo, m, err) ||
        !qindex_from_abi(qn_kind, *ket, k, err)) {
        set_error("tk_env_layout: " + err);
        return TK_ERR_INVALID_ARG;
    }
    if (3 * qn_bits(qn_kind) > 64) {
        set_error("tk_env_layout: rank-3 sector key exceeds 64 bits");
        return TK_ERR_UNSUPPORTED;
    }
    EnvLayout lay;
    env_layout(qn_kind, b, m, k, lay);
    const int64_t n = (int64_t)lay.keys.size();
    if (keys || block_offsets) {
        if (*n_blocks < n) {
            set_error("tk_env_layout: output arrays shorter than the block count");
            *n_blocks = n;
            return TK_ERR_INVALID_ARG;
        }
        for (int64_t i = 0; i < n; ++i) {
            if (keys) keys[i] = lay.keys[i];
            if (block_offsets) block_offsets[i] = lay.off[i];
        }
    }
    *n_blocks = n;
    if (total) *total = lay.total;
    return TK_OK;
}

// tk_heff2_plan_create_dev; `stacked` as in plan_create_impl (off for complex
// plans, which set their schedule once their imaginary parts are in place).
static tk_status plan_create_dev(tk_ctx* ctx, const tk_env* env_l, const tk_env* env_r, const tk_bst* w_i,
                                 const tk_bst* w_j, const int32_t* psi_flux, int32_t precision, tk_heff2_plan** out,
                                 bool stacked) {
    if (!ctx || !env_l || !env_r || !w_i || !w_j || !out || !env_l->data || !env_r->data) {
        set_error("tk_heff2_plan_create_dev: null argument");
        return TK_ERR_INVALID_ARG;
    }
    *out = nullptr;
    std::string err;
    QIndex lb, lm, lk, rb, rm, rk;
    if (!env_legs(w_i->qn_kind, *env_l, lb, lm, lk, err) || !env_legs(w_i->qn_kind, *env_r, rb, rm, rk, err)) {
        set_error("tk_heff2_plan_create_dev: environment: " + err);
        return TK_ERR_INVALID_ARG;
    }
    EnvLayout ll, rl;
    env_layout(w_i->qn_kind, lb, lm, lk, ll);
    env_layout(w_i->qn_kind, rb, rm, rk, rl);
    // the environments are small next to psi: read them once to the host to
    // build the tables and the split-precision operand stacks
    std::vector<double> lh((size_t)ll.total), rh((size_t)rl.total);
    {
        Guard g(ctx->device);
        if (!g.ok) {
            set_error("tk_heff2_plan_create_dev: cudaSetDevice failed");
            return TK_ERR_CUDA;
        }
        cudaError_t e;
        if (!lh.empty() && (e = cudaMemcpy(lh.data(), env_l->data, sizeof(double) * lh.size(), cudaMemcpyDeviceToHost)) != cudaSuccess)
            return cuda_fail("tk_heff2_plan_create_dev: read left environment", e);
        if (!rh.empty() && (e = cudaMemcpy(rh.data(), env_r->data, sizeof(double) * rh.size(), cudaMemcpyDeviceToHost)) != cudaSuccess)
            return cuda_fail("tk_heff2_plan_create_dev: read right environment", e);
    }
    return plan_create_impl(ctx, env_l, env_r, w_i, w_j, psi_flux, precision, lh.data(), rh.data(), out, stacked);
}

tk_status tk_heff2_plan_create_dev(tk_ctx* ctx, const tk_env* env_l, const tk_env* env_r, const tk_bst* w_i,
                                   const tk_bst* w_j, const int32_t* psi_flux, int32_t precision,
                                   tk_heff2_plan** out) {
    return plan_create_dev(ctx, env_l, env_r, w_i, w_j, psi_flux, precision, out, true);
}

tk_status tk_env_grow_left(tk_ctx* ctx, const tk_env* env_l, const tk_bst* a, const tk_bst* w, double* out_dev,
                           void* stream) {
    return grow("tk_env_grow_left", true, ctx, env_l, a, w, out_dev, stream);
}

tk_status tk_env_grow_right(tk_ctx* ctx, const tk_env* env_r, const tk_bst* a, const tk_bst* w, double* out_dev,
                            void* stream) {
    return grow("tk_env_grow_right", false, ctx, env_r, a, w, out_dev, stream);
}

tk_status tk_env_grow_left_complex(tk_ctx* ctx, const tk_env* env_l, const double* env_l_im, const tk_bst* a,
                                   const double* a_im, const tk_bst* w, double* out_re, double* out_im, void* stream) {
    return grow("tk_env_grow_left_complex", true, ctx, env_l, a, w, out_re, stream, env_l_im, a_im, out_im);
}

tk_status tk_env_grow_right_complex(tk_ctx* ctx, const tk_env* env_r, const double* env_r_im, const tk_bst* a,
                                    const double* a_im, const tk_bst* w, double* out_re, double* out_im, void* stream) {
    return grow("tk_env_grow_right_complex", false, ctx, env_r, a, w, out_re, stream, env_r_im, a_im, out_im);
}

tk_status tk_heff2_plan_create_dev_complex(tk_ctx* ctx, const tk_env* env_l, const double* env_l_im,
                                           const tk_env* env_r, const double* env_r_im, const tk_bst* w_i,
                                           const tk_bst* w_j, const int32_t* psi_flux, tk_heff2_plan** out) {
    if (!env_l_im || !env_r_im) {
        set_error("tk_heff2_plan_create_dev_complex: null imaginary part");
        return TK_ERR_INVALID_ARG;
    }
    tk_status st = plan_create_dev(ctx, env_l, env_r, w_i, w_j, psi_flux, TK_PREC_FP64, out, false);
    if (st != TK_OK) return st;
    tk_heff2_plan* p = *out;
    Guard g(p->device);
    cudaError_t e;
    const size_t nl = p->host.lbuf.size(), nr = p->host.rbuf.size();
    if ((e = p->lbuf_im.alloc(nl)) != cudaSuccess || (e = p->rbuf_im.alloc(nr)) != cudaSuccess ||
        (nl && (e = cudaMemcpy(p->lbuf_im.p, env_l_im, sizeof(double) * nl, cudaMemcpyDeviceToDevice)) != cudaSuccess) ||
        (nr && (e = cudaMemcpy(p->rbuf_im.p, env_r_im, sizeof(double) * nr, cudaMemcpyDeviceToDevice)) != cudaSuccess)) {
        tk_heff2_plan_destroy(p);
        *out = nullptr;
        return cuda_fail("tk_heff2_plan_create_dev_complex", e);
    }
    p->is_complex = true;
    // the complex FP64 matvec runs on operand stacks, as a real plan's does
    st = tk_heff2_set_schedule(p, TK_SCHED_STACKED);
    if (st != TK_OK) {
        tk_heff2_plan_destroy(p);
        *out = nullptr;
        return st;
    }
    return TK_OK;
}

tk_status tk_heff2_two_site_product_complex(tk_heff2_plan* plan, const tk_bst* a_i, const double* a_i_im,
                                            const tk_bst* a_j, const double* a_j_im, double* psi_re, double* psi_im,
                                            void* stream) {
    if (!plan || !a_i || !a_j || !a_i_im || !a_j_im || !psi_re || !psi_im) {
        set_error("tk_heff2_two_site_product_complex: null argument");
        return TK_ERR_INVALID_ARG;
    }
    std::string err;
    Bst3 Ai, Aj;
    if (!bst3_from_abi(*a_i, Ai, "A_i", err) || !bst3_from_abi(*a_j, Aj, "A_j", err)) {
        set_error("tk_heff2_two_site_product_complex: " + err);
        return TK_ERR_INVALID_ARG;
    }
    GemmTable gt;
    tk_status st = build_product_tables(plan->host, Ai, Aj, gt, err);
    if (st != TK_OK) {
        set_error("tk_heff2_two_site_product_complex: " + err);
        return st;
    }
    Guard gd(plan->device);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e;
    const size_t n = (size_t)plan->host.total;
    if ((e = cudaMemsetAsync(psi_re, 0, sizeof(double) * n, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(psi_im, 0, sizeof(double) * n, s)) != cudaSuccess)
        return cuda_fail("cudaMemsetAsync", e);
    Scratch sc(s);
    DevTable g;
    if ((st = g.upload(sc, gt)) != TK_OK) return st;
    if ((e = launch_gemm_c64(g.tl, g.n, g.t, g.sg, Ai.data, a_i_im, Aj.data, a_j_im, psi_re, psi_im, false, s)) !=
        cudaSuccess)
        return cuda_fail("grouped gemm", e);
    return TK_OK;
}

tk_status tk_heff2_two_site_product(tk_heff2_plan* plan, const tk_bst* a_i, const tk_bst* a_j, double* psi_dev,
                                    void* stream) {
    if (!plan || !a_i || !a_j || !psi_dev) {
        set_error("tk_heff2_two_site_product: null argument");
        return TK_ERR_INVALID_ARG;
    }
    std::string err;
    Bst3 Ai, Aj;
    if (!bst3_from_abi(*a_i, Ai, "A_i", err) || !bst3_from_abi(*a_j, Aj, "A_j", err)) {
        set_error("tk_heff2_two_site_product: " + err);
        return TK_ERR_INVALID_ARG;
    }
    GemmTable g;
    tk_status st = build_product_tables(plan->host, Ai, Aj, g, err);
    if (st != TK_OK) {
        set_error("tk_heff2_two_site_product: " + err);
        return st;
    }
    Guard gd(plan->device);
    if (!gd.ok) {
        set_error("tk_heff2_two_site_product: cudaSetDevice failed");
        return TK_ERR_CUDA;
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e;
    if ((e = cudaMemsetAsync(psi_dev, 0, sizeof(double) * (size_t)plan->host.total, s)) != cudaSuccess)
        return cuda_fail("cudaMemsetAsync", e);
    Scratch sc(s);
    return launch_table(sc, g, Ai.data, Aj.data, psi_dev);
}

}  // extern "C"
