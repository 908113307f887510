// tk_bsgemm.hpp -- rank-2 block-sparse GEMM planning shared by block_gemm
// and the pairwise contraction.
//
// Task rules of SparseLinAlgBackend::block_gemm
// (tk-linalg/src/device/faer.rs:390-575, tk-linalg/src/tasks.rs:36-81,180-188):
// a task for every (key_a, key_b) pair whose contracted quantum numbers are
// equal (A's column charge == B's row charge) and whose output sector
// satisfies row (+) dual(col) == flux_a (+) flux_b; contributions to one
// output key are summed (here in registers: one output block per task, its
// K dimension a list of segments); output keys ascending; output legs
// [a.legs[0], b.legs[1]] with directions [a.dirs[0], b.dirs[1]].
#pragma once
#include <map>
#include <string>
#include <vector>

#include "tk_internal.hpp"

namespace tk {

// A rank-2 block-sparse tensor as the GEMM sees it: legs, directions, flux,
// keys ascending with the sector index of each block on both legs, block
// offsets into one buffer (host or device: `data` is not read here).
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

inline bool rank2_from_abi(const tk_bst& t, Rank2& o, const char* name, std::string& err) {
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
        if (t.block_offsets[b] < 0) {
            err = std::string(name) + ": negative block offset";
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

// The output layout and the grouped-GEMM tables of C = A B.
struct BlockGemmPlan {
    GemmTable g;
    std::vector<uint64_t> okeys;
    std::vector<int64_t> ooffs;
    int64_t total = 0;
    Qn target;
};

inline void bsgemm_tiles_for(GemmTable& g, int task) {
    const GemmTask& t = g.tasks[task];
    for (int m0 = 0; m0 < t.M; m0 += 64)
        for (int n0 = 0; n0 < t.N; n0 += 64) g.tiles.push_back({task, m0, n0, 0});
}

// Smaller square tiles for small products.  With fewer 64 x 64 tiles than
// the GPU holds, most SMs would sit idle while a few run a whole tile over
// the full K (this GPU's FP64 pipe retires two FMAs per clock per SM, so one
// 64 x 64 x 130 tile is ~0.13 ms on one SM): the tasks whose tiles are the
// heaviest (edge^2 x K) go to the next smaller edge (32, then 16) until there
// are `target` tiles or every task is at the smallest edge; then the tiles
// go out longest first.  Each output element still comes from one tile that
// sums the task's segments in the same order.
inline void bsgemm_retile(GemmTable& g, size_t target) {
    const size_t nt = g.tasks.size();
    std::vector<int> cls(nt, 0);
    std::vector<double> ktot(nt, 0.0);
    for (size_t t = 0; t < nt; ++t)
        for (int s = g.tasks[t].seg_begin; s < g.tasks[t].seg_end; ++s) ktot[t] += g.segs[(size_t)s].K;
    auto ntiles = [&](size_t t, int c) {
        const int e = 64 >> c;
        return (size_t)((g.tasks[t].M + e - 1) / e) * (size_t)((g.tasks[t].N + e - 1) / e);
    };
    size_t total = 0;
    for (size_t t = 0; t < nt; ++t) total += ntiles(t, 0);
    while (total < target) {
        size_t best = nt;
        double best_cost = 0.0;
        for (size_t t = 0; t < nt; ++t) {
            if (cls[t] + 1 >= kGemmTileClasses) continue;
            const double e = (double)(64 >> cls[t]);
            const double c = e * e * ktot[t];
            if (best == nt || c > best_cost) {
                best = t;
                best_cost = c;
            }
        }
        if (best == nt) break;
        total += ntiles(best, cls[best] + 1) - ntiles(best, cls[best]);
        ++cls[best];
    }
    g.tiles.clear();
    for (size_t t = 0; t < nt; ++t) {
        const int e = 64 >> cls[t];
        for (int m0 = 0; m0 < g.tasks[t].M; m0 += e)
            for (int n0 = 0; n0 < g.tasks[t].N; n0 += e) g.tiles.push_back({(int)t, m0, n0, cls[t]});
    }
    gemm_lpt_order(g, 64, 64);
}

// TK_OK, TK_ERR_INVALID_ARG (kinds differ) or TK_ERR_SECTOR_MISMATCH
// (matched contracted sectors of different dimensions), with `err` set.
inline tk_status block_gemm_plan(const Rank2& A, const Rank2& B, BlockGemmPlan& P, std::string& err) {
    if (A.kind != B.kind) {
        err = "quantum-number kinds differ";
        return TK_ERR_INVALID_ARG;
    }
    const int kind = A.kind;
    P.target = qn_fuse(kind, A.flux, B.flux);
    // phase 1 (faer.rs:406-430): a task per compatible pair
    std::map<uint64_t, std::vector<std::pair<int, int>>> by_out;
    for (size_t i = 0; i < A.keys.size(); ++i)
        for (size_t j = 0; j < B.keys.size(); ++j) {
            const Qn& qa_col = A.legs[1].q[A.cs[i]];
            const Qn& qb_row = B.legs[0].q[B.rs[j]];
            if (qa_col != qb_row) continue;
            Qn out_q[2] = {A.legs[0].q[A.rs[i]], B.legs[1].q[B.cs[j]]};
            if (qn_fuse(kind, out_q[0], qn_dual(kind, out_q[1])) != P.target) continue;
            if (A.legs[1].dim[A.cs[i]] != B.legs[0].dim[B.rs[j]]) {
                err = "contracted sector dimensions differ";
                return TK_ERR_SECTOR_MISMATCH;
            }
            by_out[key_pack(kind, out_q, 2)].push_back({(int)i, (int)j});
        }
    // output blocks in ascending key order (faer.rs:560-574)
    P.total = 0;
    for (auto& kv : by_out) {
        const auto& pairs = kv.second;
        int i0 = pairs[0].first, j0 = pairs[0].second;
        int64_t M = A.legs[0].dim[A.rs[i0]], N = B.legs[1].dim[B.cs[j0]];
        GemmTask t{};
        t.M = (int32_t)M;
        t.N = (int32_t)N;
        t.c_off = P.total;
        t.c_rs = (int32_t)N;
        t.c_cs = 1;
        t.alpha = 1.0;
        t.beta = 0.0;
        t.seg_begin = (int)P.g.segs.size();
        for (auto& pr : pairs) {
            int64_t K = A.legs[1].dim[A.cs[pr.first]];
            GemmSeg s{};
            s.a_off = A.offs[pr.first];
            s.a_rs = (int32_t)K;
            s.a_cs = 1;
            s.b_off = B.offs[pr.second];
            s.b_rs = (int32_t)N;
            s.b_cs = 1;
            s.K = (int32_t)K;
            P.g.segs.push_back(s);
            P.g.flops += 2.0 * M * N * K;
        }
        t.seg_end = (int)P.g.segs.size();
        P.g.tasks.push_back(t);
        bsgemm_tiles_for(P.g, (int)P.g.tasks.size() - 1);
        P.okeys.push_back(kv.first);
        P.ooffs.push_back(P.total);
        P.total += M * N;
    }
    bsgemm_retile(P.g, 2 * 152);
    return TK_OK;
}

}  // namespace tk
