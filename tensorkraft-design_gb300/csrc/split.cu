// split.cu -- the two-site truncation's data path on the device.
//
// After the eigensolver, DMRGEngine::dmrg_step_two_site (tk-dmrg/src/sweep/
// mod.rs:398-437) truncates the two-site vector with truncate_svd
// (tk-dmrg/src/truncation/mod.rs:56-127).  With U(1)-type charges the
// two-site matrix M[(s_i, a_L), (s_j, a_R)] is block diagonal in the bond
// charge q = q(s_i) + q(a_L) = q(a_R) - q(s_j), so its SVD is the SVD of every
// block M_q.  This file moves the data on the device, where psi already is:
//   * tk_split_gather: every psi sub-block copied into its M_q (one launch,
//     all charges packed back to back, row-major), then one copy to the host,
//     whose LAPACK decomposes each M_q (the reference hands its SVD to faer on
//     the host as well; this GPU's FP64 rate is no higher than the host's for
//     these many small factorisations);
//   * tk_split_factors: the kept columns of U and rows of V^T (scaled by the
//     caller) copied up once and scattered straight into the new site
//     tensors' block layouts (one launch per factor).
// The caller applies truncate_svd's rule to the singular values of all
// charges between the two calls.
//
// Row groups of M_q: (s_i state, a_L sector), states ascending then sectors
// ascending; column groups (s_j state, a_R sector) likewise.  New site
// tensors: A_i (s_i, a_L, bond) with blocks (q_s, q_a, q), A_j (s_j, bond,
// a_R) with blocks (q_s, q, q_b), each FlatBlockStorage (keys ascending,
// row-major blocks), bond = the kept charges ascending.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "tk_internal.hpp"
#include "tk_plan.cuh"

namespace tk {
namespace {

// One strided rectangle copy: dst[dst_off + r * dst_rs + c * dst_cs] =
// src[src_off + r * src_rs + c * src_cs], r < rows, c < cols.
struct CopySeg {
    int64_t src_off, dst_off;
    int32_t rows, cols, src_rs, src_cs, dst_rs, dst_cs;
};

__global__ void copy_segs_kernel(const CopySeg* __restrict__ segs, const double* __restrict__ src,
                                 double* __restrict__ dst) {
    const CopySeg g = segs[blockIdx.y];
    const int n = g.rows * g.cols;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int r = e / g.cols, c = e - r * g.cols;
        dst[g.dst_off + (int64_t)r * g.dst_rs + (int64_t)c * g.dst_cs] =
            src[g.src_off + (int64_t)r * g.src_rs + (int64_t)c * g.src_cs];
    }
}

cudaError_t launch_copy(const CopySeg* d_segs, int nseg, int max_elems, const double* src, double* dst,
                        cudaStream_t s) {
    if (nseg <= 0) return cudaSuccess;
    for (int y0 = 0; y0 < nseg; y0 += 65535) {
        const int ny = std::min(65535, nseg - y0);
        dim3 grid((unsigned)std::max(1, std::min((max_elems + 255) / 256, 32)), (unsigned)ny);
        copy_segs_kernel<<<grid, 256, 0, s>>>(d_segs + y0, src, dst);
    }
    return cudaGetLastError();
}

struct Group {
    int state_sec;   // physical sector of the state
    int64_t local;   // index of the state inside its sector
    int sec;         // bond sector (a_L for rows, a_R for columns)
    int64_t off;     // offset inside M_q (row or column)
};

struct Charge {
    Qn q;
    std::vector<Group> rows, cols;
    int64_t m = 0, n = 0;     // M_q is m x n
    int64_t moff = 0;         // offset of M_q in the packed buffer (row-major m x n)
    int64_t kept = 0, uoff = 0, voff = 0;  // U_q (m x kept) and V_q (kept x n) in the factor packs
};

}  // namespace
}  // namespace tk

struct tk_split_plan {
    tk_ctx* ctx = nullptr;
    int kind = 0;
    tk::QIndex legs[4];
    std::vector<tk::Charge> ch;
    int64_t m_total = 0;
    std::vector<tk::CopySeg> gather;   // psi -> packed M
    int gather_max = 0;
    // kept-set dependent: layouts and scatter segments
    std::vector<uint64_t> keys_i, keys_j;
    std::vector<int64_t> offs_i, offs_j;
    int64_t total_i = 0, total_j = 0, u_total = 0, v_total = 0;
    std::vector<tk::CopySeg> scat_u, scat_v;
    int scat_u_max = 0, scat_v_max = 0;
    bool have_kept = false;
};

using namespace tk;

namespace {

struct DevGuard {
    int prev = -1;
    explicit DevGuard(int d) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        cudaSetDevice(d);
    }
    ~DevGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

#define CKS(op)                                          \
    do {                                                 \
        cudaError_t e_ = (op);                           \
        if (e_ != cudaSuccess) return cuda_fail(#op, e_); \
    } while (0)

tk_status split_build(tk_split_plan& S, const int64_t n_blocks, const uint64_t* keys, const int64_t* offsets,
                      std::string& err) {
    const int kind = S.kind;
    const QIndex &PI = S.legs[0], &PJ = S.legs[1], &QA = S.legs[2], &QB = S.legs[3];
    // charges: rows (s_i state, A) and columns (s_j state, B)
    std::map<std::pair<int32_t, int32_t>, Charge> by;
    for (int ps = 0; ps < PI.n(); ++ps)
        for (int64_t l = 0; l < PI.dim[ps]; ++l)
            for (int a = 0; a < QA.n(); ++a) {
                const Qn q = qn_fuse(kind, PI.q[ps], QA.q[a]);
                Charge& c = by[{q.c[0], q.c[1]}];
                c.q = q;
                c.rows.push_back({ps, l, a, c.m});
                c.m += QA.dim[a];
            }
    for (int ps = 0; ps < PJ.n(); ++ps)
        for (int64_t l = 0; l < PJ.dim[ps]; ++l)
            for (int b = 0; b < QB.n(); ++b) {
                const Qn q = qn_fuse(kind, QB.q[b], qn_dual(kind, PJ.q[ps]));
                auto it = by.find({q.c[0], q.c[1]});
                if (it == by.end()) continue;  // no row of that charge
                Charge& c = it->second;
                c.cols.push_back({ps, l, b, c.n});
                c.n += QB.dim[b];
            }
    // charges with rows and columns, ascending (qn order)
    for (auto& kv : by)
        if (kv.second.m > 0 && kv.second.n > 0) S.ch.push_back(std::move(kv.second));
    std::sort(S.ch.begin(), S.ch.end(), [](const Charge& a, const Charge& b) { return qn_less(a.q, b.q); });
    std::map<std::pair<int32_t, int32_t>, int> cpos;
    for (size_t i = 0; i < S.ch.size(); ++i) cpos[{S.ch[i].q.c[0], S.ch[i].q.c[1]}] = (int)i;
    S.m_total = 0;
    for (Charge& c : S.ch) {
        c.moff = S.m_total;
        S.m_total += c.m * c.n;
    }
    // row / column group lookup per charge: (state sector, local, bond sector) -> offset
    std::vector<std::map<std::tuple<int, int64_t, int>, int64_t>> roff(S.ch.size()), coff(S.ch.size());
    for (size_t i = 0; i < S.ch.size(); ++i) {
        for (const Group& g : S.ch[i].rows) roff[i][{g.state_sec, g.local, g.sec}] = g.off;
        for (const Group& g : S.ch[i].cols) coff[i][{g.state_sec, g.local, g.sec}] = g.off;
    }
    // gather: every psi sub-block (li, lj) of every block into its M_q
    for (int64_t b = 0; b < n_blocks; ++b) {
        Qn q[4];
        key_unpack(kind, keys[b], 4, q);
        const int si = PI.find(q[0]), sj = PJ.find(q[1]), a = QA.find(q[2]), bb = QB.find(q[3]);
        if (si < 0 || sj < 0 || a < 0 || bb < 0) {
            err = "two-site block key names a sector missing from its leg";
            return TK_ERR_INVALID_ARG;
        }
        const Qn qr = qn_fuse(kind, q[0], q[2]);
        auto it = cpos.find({qr.c[0], qr.c[1]});
        if (it == cpos.end()) {
            err = "two-site block outside the flux-zero charge structure";
            return TK_ERR_SECTOR_MISMATCH;
        }
        const int ci = it->second;
        const Charge& c = S.ch[ci];
        const int64_t DA = QA.dim[a], DB = QB.dim[bb], ni = PI.dim[si], nj = PJ.dim[sj];
        for (int64_t li = 0; li < ni; ++li)
            for (int64_t lj = 0; lj < nj; ++lj) {
                auto r = roff[ci].find({si, li, a});
                auto k = coff[ci].find({sj, lj, bb});
                if (r == roff[ci].end() || k == coff[ci].end()) {
                    err = "two-site block outside the flux-zero charge structure";
                    return TK_ERR_SECTOR_MISMATCH;
                }
                CopySeg g{};
                g.src_off = offsets[b] + (li * nj + lj) * DA * DB;
                g.dst_off = c.moff + r->second * c.n + k->second;
                g.rows = (int32_t)DA;
                g.cols = (int32_t)DB;
                g.src_rs = (int32_t)DB;
                g.src_cs = 1;
                g.dst_rs = (int32_t)c.n;
                g.dst_cs = 1;
                S.gather.push_back(g);
                S.gather_max = std::max<int>(S.gather_max, (int)(DA * DB));
            }
    }
    if (S.m_total > INT32_MAX * 64ll || S.gather.size() > (size_t)INT32_MAX) {
        err = "two-site vector too large for the split tables";
        return TK_ERR_UNSUPPORTED;
    }
    return TK_OK;
}

// Layouts of A_i / A_j for the kept counts and the scatters of the factor packs.
tk_status split_set_kept(tk_split_plan& S, const int64_t* kept, std::string& err) {
    const int kind = S.kind;
    const QIndex &PI = S.legs[0], &PJ = S.legs[1], &QA = S.legs[2], &QB = S.legs[3];
    S.u_total = S.v_total = 0;
    for (size_t i = 0; i < S.ch.size(); ++i) {
        Charge& c = S.ch[i];
        if (kept[i] < 0 || kept[i] > std::min(c.m, c.n)) {
            err = "kept count out of range for its charge";
            return TK_ERR_INVALID_ARG;
        }
        c.kept = kept[i];
        c.uoff = S.u_total;
        S.u_total += c.m * c.kept;
        c.voff = S.v_total;
        S.v_total += c.kept * c.n;
    }
    // blocks of A_i (q_s, q_a, q) and A_j (q_s, q, q_b), keys ascending
    struct Blk {
        uint64_t key;
        int ci, ps, sec;   // charge, physical sector, bond sector
        int64_t size;
    };
    std::vector<Blk> bi, bj;
    for (size_t i = 0; i < S.ch.size(); ++i) {
        const Charge& c = S.ch[i];
        if (c.kept == 0) continue;
        std::map<std::pair<int, int>, bool> seen;
        for (const Group& g : c.rows)
            if (!seen[{g.state_sec, g.sec}]) {
                seen[{g.state_sec, g.sec}] = true;
                Qn q[3] = {PI.q[g.state_sec], QA.q[g.sec], c.q};
                bi.push_back({key_pack(kind, q, 3), (int)i, g.state_sec, g.sec, PI.dim[g.state_sec] * QA.dim[g.sec] * c.kept});
            }
        seen.clear();
        for (const Group& g : c.cols)
            if (!seen[{g.state_sec, g.sec}]) {
                seen[{g.state_sec, g.sec}] = true;
                Qn q[3] = {PJ.q[g.state_sec], c.q, QB.q[g.sec]};
                bj.push_back({key_pack(kind, q, 3), (int)i, g.state_sec, g.sec, PJ.dim[g.state_sec] * c.kept * QB.dim[g.sec]});
            }
    }
    auto by_key = [](const Blk& a, const Blk& b) { return a.key < b.key; };
    std::sort(bi.begin(), bi.end(), by_key);
    std::sort(bj.begin(), bj.end(), by_key);
    std::map<std::tuple<int, int, int>, int64_t> ioff, joff;  // (charge, phys sector, bond sector) -> block offset
    S.keys_i.clear(); S.offs_i.clear(); S.keys_j.clear(); S.offs_j.clear();
    S.total_i = S.total_j = 0;
    for (const Blk& b : bi) {
        S.keys_i.push_back(b.key);
        S.offs_i.push_back(S.total_i);
        ioff[{b.ci, b.ps, b.sec}] = S.total_i;
        S.total_i += b.size;
    }
    for (const Blk& b : bj) {
        S.keys_j.push_back(b.key);
        S.offs_j.push_back(S.total_j);
        joff[{b.ci, b.ps, b.sec}] = S.total_j;
        S.total_j += b.size;
    }
    // one segment per (state, bond sector) group: A_i[l][a][kk] = U_q[g.off + a][kk],
    // A_j[l][kk][b] = V_q[kk][g.off + b]
    S.scat_u.clear(); S.scat_v.clear();
    S.scat_u_max = S.scat_v_max = 0;
    for (size_t i = 0; i < S.ch.size(); ++i) {
        const Charge& c = S.ch[i];
        if (c.kept == 0) continue;
        const int32_t k = (int32_t)c.kept;
        for (const Group& g : c.rows) {
            const int64_t D = QA.dim[g.sec];
            CopySeg sg{};
            sg.src_off = c.uoff + g.off * k; sg.src_rs = k; sg.src_cs = 1;
            sg.dst_off = ioff.at({(int)i, g.state_sec, g.sec}) + g.local * D * k;
            sg.rows = (int32_t)D; sg.cols = k; sg.dst_rs = k; sg.dst_cs = 1;
            S.scat_u.push_back(sg);
            S.scat_u_max = std::max<int>(S.scat_u_max, (int)(D * k));
        }
        for (const Group& g : c.cols) {
            const int64_t D = QB.dim[g.sec];
            CopySeg sg{};
            sg.src_off = c.voff + g.off; sg.src_rs = (int32_t)c.n; sg.src_cs = 1;
            sg.dst_off = joff.at({(int)i, g.state_sec, g.sec}) + g.local * k * D;
            sg.rows = k; sg.cols = (int32_t)D; sg.dst_rs = (int32_t)D; sg.dst_cs = 1;
            S.scat_v.push_back(sg);
            S.scat_v_max = std::max<int>(S.scat_v_max, (int)(D * k));
        }
    }
    S.have_kept = true;
    return TK_OK;
}

tk_status fail_s(const std::string& m, tk_status c) {
    set_error(m);
    return c;
}

}  // namespace

extern "C" {

tk_status tk_split_plan_create(tk_ctx* ctx, int32_t qn_kind, const tk_qindex* legs, int64_t n_blocks,
                               const uint64_t* keys, const int64_t* offsets, tk_split_plan** out) {
    if (!ctx || !legs || !out || (n_blocks > 0 && (!keys || !offsets)) || n_blocks < 0)
        return fail_s("tk_split_plan_create: invalid argument", TK_ERR_INVALID_ARG);
    *out = nullptr;
    if (!qn_kind_valid(qn_kind) || 4 * qn_bits(qn_kind) > 64)
        return fail_s("tk_split_plan_create: unknown quantum-number kind", TK_ERR_INVALID_ARG);
    std::unique_ptr<tk_split_plan> S(new (std::nothrow) tk_split_plan);
    if (!S) return fail_s("tk_split_plan_create: host allocation failed", TK_ERR_OOM);
    S->ctx = ctx;
    S->kind = qn_kind;
    std::string err;
    for (int l = 0; l < 4; ++l)
        if (!qindex_from_abi(qn_kind, legs[l], S->legs[l], err))
            return fail_s("tk_split_plan_create: " + err, TK_ERR_INVALID_ARG);
    tk_status st = guard_host("tk_split_plan_create", err, [&] { return split_build(*S, n_blocks, keys, offsets, err); });
    if (st != TK_OK) return fail_s("tk_split_plan_create: " + err, st);
    *out = S.release();
    return TK_OK;
}

void tk_split_plan_destroy(tk_split_plan* s) {
    if (!s) return;
    DevGuard g(s->ctx->device);
    delete s;
}

tk_status tk_split_charges(const tk_split_plan* s, int32_t* n_charges, int32_t* charges, int64_t* rows, int64_t* cols) {
    if (!s || !n_charges) return fail_s("tk_split_charges: invalid argument", TK_ERR_INVALID_ARG);
    *n_charges = (int32_t)s->ch.size();
    const int nc = qn_ncomp(s->kind);
    for (size_t i = 0; i < s->ch.size(); ++i) {
        if (charges)
            for (int k = 0; k < nc; ++k) charges[i * nc + k] = s->ch[i].q.c[k];
        if (rows) rows[i] = s->ch[i].m;
        if (cols) cols[i] = s->ch[i].n;
    }
    return TK_OK;
}

tk_status tk_split_gather(tk_split_plan* s, const double* psi_dev, double* m_host, void* stream) {
    if (!s || !psi_dev || (!m_host && s->m_total > 0)) return fail_s("tk_split_gather: invalid argument", TK_ERR_INVALID_ARG);
    if (s->m_total == 0) return TK_OK;
    DevGuard g(s->ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    Blob blob;
    const size_t og = blob.add(s->gather.data(), sizeof(CopySeg) * s->gather.size());
    const size_t om = blob.reserve(sizeof(double) * (size_t)s->m_total);
    void *dv = nullptr, *hv = nullptr;
    tk_status r;
    if ((r = ctx_dev_scratch(s->ctx, blob.device_size(), &dv)) != TK_OK) return r;
    if ((r = ctx_host_stage(s->ctx, std::max<size_t>(blob.size(), 1), &hv)) != TK_OK) return r;
    unsigned char* d = static_cast<unsigned char*>(dv);
    blob.copy_to(hv);
    double* m = (double*)(d + om);
    CKS(cudaMemcpyAsync(d, hv, blob.size(), cudaMemcpyHostToDevice, st));
    // elements of M_q that no psi block reaches are zero
    CKS(cudaMemsetAsync(m, 0, sizeof(double) * (size_t)s->m_total, st));
    CKS(launch_copy((const CopySeg*)(d + og), (int)s->gather.size(), s->gather_max, psi_dev, m, st));
    CKS(cudaMemcpyAsync(m_host, m, sizeof(double) * (size_t)s->m_total, cudaMemcpyDeviceToHost, st));
    CKS(cudaStreamSynchronize(st));
    return TK_OK;
}

tk_status tk_split_set_kept(tk_split_plan* s, const int64_t* kept, int64_t* n_blocks_i, int64_t* total_i,
                            int64_t* n_blocks_j, int64_t* total_j) {
    if (!s || (!kept && !s->ch.empty())) return fail_s("tk_split_set_kept: invalid argument", TK_ERR_INVALID_ARG);
    std::string err;
    tk_status st = guard_host("tk_split_set_kept", err, [&] { return split_set_kept(*s, kept, err); });
    if (st != TK_OK) return fail_s("tk_split_set_kept: " + err, st);
    if (n_blocks_i) *n_blocks_i = (int64_t)s->keys_i.size();
    if (total_i) *total_i = s->total_i;
    if (n_blocks_j) *n_blocks_j = (int64_t)s->keys_j.size();
    if (total_j) *total_j = s->total_j;
    return TK_OK;
}

tk_status tk_split_layout(const tk_split_plan* s, int32_t side, uint64_t* keys, int64_t* offsets) {
    if (!s || !s->have_kept || (side != 0 && side != 1))
        return fail_s("tk_split_layout: invalid argument (set the kept counts first)", TK_ERR_INVALID_ARG);
    const auto& k = side == 0 ? s->keys_i : s->keys_j;
    const auto& o = side == 0 ? s->offs_i : s->offs_j;
    if (keys) std::copy(k.begin(), k.end(), keys);
    if (offsets) std::copy(o.begin(), o.end(), offsets);
    return TK_OK;
}

tk_status tk_split_factors(tk_split_plan* s, const double* u_host, const double* v_host, double* ai_dev,
                           double* aj_dev, void* stream) {
    if (!s || !s->have_kept || (s->u_total > 0 && (!u_host || !v_host)) || (s->total_i > 0 && !ai_dev) ||
        (s->total_j > 0 && !aj_dev))
        return fail_s("tk_split_factors: invalid argument (tk_split_set_kept first)", TK_ERR_INVALID_ARG);
    if (s->u_total == 0) return TK_OK;
    DevGuard g(s->ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    Blob blob;
    const size_t ou = blob.add(u_host, sizeof(double) * (size_t)s->u_total);
    const size_t ov = blob.add(v_host, sizeof(double) * (size_t)s->v_total);
    const size_t osu = blob.add(s->scat_u.data(), sizeof(CopySeg) * s->scat_u.size());
    const size_t osv = blob.add(s->scat_v.data(), sizeof(CopySeg) * s->scat_v.size());
    void *dv = nullptr, *hv = nullptr;
    tk_status r;
    if ((r = ctx_dev_scratch(s->ctx, blob.device_size(), &dv)) != TK_OK) return r;
    if ((r = ctx_host_stage(s->ctx, std::max<size_t>(blob.size(), 1), &hv)) != TK_OK) return r;
    unsigned char* d = static_cast<unsigned char*>(dv);
    blob.copy_to(hv);
    CKS(cudaMemcpyAsync(d, hv, blob.size(), cudaMemcpyHostToDevice, st));
    CKS(launch_copy((const CopySeg*)(d + osu), (int)s->scat_u.size(), s->scat_u_max, (const double*)(d + ou), ai_dev, st));
    CKS(launch_copy((const CopySeg*)(d + osv), (int)s->scat_v.size(), s->scat_v_max, (const double*)(d + ov), aj_dev, st));
    // the packs live in the context's shared scratch: finish before returning
    CKS(cudaStreamSynchronize(st));
    return TK_OK;
}

}  // extern "C"
