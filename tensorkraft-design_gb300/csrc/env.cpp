// env.cpp -- host tables for block-sparse environments on the device.
//
// Environment growth by one site restates contract_left_environment and
// contract_right_environment (tk-dmrg/src/environments/mod.rs:221-483):
//   L'[b', v, b] = sum conj(A[s', a', b']) L[a', w, a] W[s, s', w, v] A[s, a, b]
//   R'[a', w, a] = sum conj(A[s', a', b']) R[b', v, b] W[s, s', w, v] A[s, a, b]
// (W's first leg s_in pairs with the ket A, its second s_out with the bra).
// The reference loops over every (ket block, bra block, MPO block) triple
// into a dense (bra, w, ket) array; here both environments are block-sparse
// in the canonical layout (only sector triples with q(bra) = q(ket) + q(w)
// exist, which is where a symmetric environment is non-zero) and the
// contraction is three launches over flat tables:
//   stage 1  grouped GEMM   T1 = L * A        (left)   A * R^T  (right)
//   stage 2  channel combine T2 = W (x) T1
//   stage 3  grouped GEMM   L' = A^T * T2     (left)   A * T2^T (right)
// The two-site start vector psi(s_i, s_j, a, b) = sum_c A_i(s_i, a, c) A_j(s_j, c, b)
// in a plan's block layout is one more grouped GEMM.
#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "tk_env.hpp"

namespace tk {

void env_layout(int kind, const QIndex& bra, const QIndex& mpo, const QIndex& ket, EnvLayout& out) {
    out = EnvLayout();
    std::vector<std::pair<uint64_t, std::array<int, 3>>> kb;
    for (int b = 0; b < bra.n(); ++b)
        for (int w = 0; w < mpo.n(); ++w) {
            // q(ket) = q(bra) - q(w)
            Qn qk = qn_fuse(kind, bra.q[b], qn_dual(kind, mpo.q[w]));
            int k = ket.find(qk);
            if (k < 0) continue;
            Qn q3[3] = {bra.q[b], mpo.q[w], ket.q[k]};
            kb.push_back({key_pack(kind, q3, 3), {b, w, k}});
        }
    std::sort(kb.begin(), kb.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
    int64_t off = 0;
    for (const auto& e : kb) {
        out.keys.push_back(e.first);
        out.tri.push_back(e.second);
        out.off.push_back(off);
        off += bra.dim[e.second[0]] * mpo.dim[e.second[1]] * ket.dim[e.second[2]];
    }
    out.total = off;
}

bool bst3_from_abi(const tk_bst& t, Bst3& o, const char* name, std::string& err) {
    if (t.rank != 3 || !t.legs) {
        err = std::string(name) + ": MPS site tensor must have rank 3 (s, a_L, a_R)";
        return false;
    }
    if (!qn_kind_valid(t.qn_kind)) {
        err = std::string(name) + ": unknown quantum-number kind";
        return false;
    }
    o.kind = t.qn_kind;
    for (int l = 0; l < 3; ++l)
        if (!qindex_from_abi(t.qn_kind, t.legs[l], o.legs[l], err)) {
            err = std::string(name) + ": " + err;
            return false;
        }
    if (t.n_blocks < 0 || (t.n_blocks > 0 && (!t.keys || !t.block_offsets || !t.data))) {
        err = std::string(name) + ": null block arrays";
        return false;
    }
    o.data = t.data;
    const QIndex& P = o.legs[0];
    const QIndex& QL = o.legs[1];
    o.blk.assign((size_t)P.n() * QL.n(), -1);
    o.right.assign((size_t)P.n() * QL.n(), -1);
    int64_t end = 0;
    for (int64_t b = 0; b < t.n_blocks; ++b) {
        if (b > 0 && t.keys[b - 1] >= t.keys[b]) {
            err = std::string(name) + ": sector keys not strictly ascending";
            return false;
        }
        Qn q[3];
        key_unpack(o.kind, t.keys[b], 3, q);
        int s = P.find(q[0]), l = QL.find(q[1]), r = o.legs[2].find(q[2]);
        if (s < 0 || l < 0 || r < 0) {
            err = std::string(name) + ": block key names a sector missing from its QIndex";
            return false;
        }
        if (qn_fuse(o.kind, q[0], q[1]) != q[2]) {
            err = std::string(name) + ": block violates q(s) + q(a_L) = q(a_R)";
            return false;
        }
        if (t.block_offsets[b] < end) {
            err = std::string(name) + ": block offsets overlap";
            return false;
        }
        o.blk[(size_t)s * QL.n() + l] = t.block_offsets[b];
        o.right[(size_t)s * QL.n() + l] = r;
        end = t.block_offsets[b] + P.dim[s] * QL.dim[l] * o.legs[2].dim[r];
    }
    o.total = end;
    return true;
}

namespace {

// physical state -> (sector, local index)
void state_map(const QIndex& P, std::vector<int>& sec, std::vector<int64_t>& loc) {
    sec.assign(P.total, 0);
    loc.assign(P.total, 0);
    for (int s = 0; s < P.n(); ++s)
        for (int64_t k = 0; k < P.dim[s]; ++k) {
            sec[P.off[s] + k] = s;
            loc[P.off[s] + k] = k;
        }
}

// Offset of the (D_L x D_R) sub-block of physical state `st` in the block of
// (sector(st), left sector l), or -1.
int64_t site_sub(const Bst3& A, const std::vector<int>& ssec, const std::vector<int64_t>& sloc, int64_t st, int l,
                 int* r_out) {
    const int nl = A.legs[1].n();
    const int s = ssec[st];
    const int64_t b = A.blk[(size_t)s * nl + l];
    if (b < 0) return -1;
    const int r = A.right[(size_t)s * nl + l];
    *r_out = r;
    return b + sloc[st] * A.legs[1].dim[l] * A.legs[2].dim[r];
}

bool finish(GrowTables& G, int64_t n_env, int64_t n_site, int64_t n_out, bool left, std::string& err) {
    gemm_lpt_order(G.g1, kEnvTileM, kEnvTileN);
    gemm_lpt_order(G.g3, kEnvTileM, kEnvTileN);
    if (G.g1.tiles.size() > (size_t)INT32_MAX || G.g3.tiles.size() > (size_t)INT32_MAX ||
        G.jobs.size() > (size_t)INT32_MAX || G.terms.size() > (size_t)INT32_MAX) {
        err = "environment tables exceed 32-bit index range";
        return false;
    }
    // stage 1 reads (env, site) [left] or (site, env) [right]; stage 3 reads (site, T2)
    if (left ? !gemm_table_ok(G.g1, n_env, n_site, G.t1_total, "env stage 1", err)
             : !gemm_table_ok(G.g1, n_site, n_env, G.t1_total, "env stage 1", err))
        return false;
    if (!comb_table_ok(G.jobs, G.terms, G.t1_total, G.t2_total, err)) return false;
    if (!gemm_table_ok(G.g3, n_site, G.t2_total, n_out, "env stage 3", err)) return false;
    return true;
}

}  // namespace

static tk_status build_grow_tables_body(bool left, const QIndex& env_bra, const QIndex& env_mpo,
                                        const QIndex& env_ket, const Bst3& A, const Bst4& W, GrowTables& G,
                                        std::string& err) {
    G = GrowTables();
    const int kind = A.kind;
    const QIndex& P = A.legs[0];
    const QIndex& QL = A.legs[1];
    const QIndex& QR = A.legs[2];
    if (!env_bra.same_as(env_ket)) {
        err = "environment bra and ket QIndex differ";
        return TK_ERR_SECTOR_MISMATCH;
    }
    if (!W.legs[0].same_as(P) || !W.legs[1].same_as(P)) {
        err = "MPO physical legs differ from the MPS physical leg";
        return TK_ERR_SECTOR_MISMATCH;
    }
    // left: the environment sits on the MPS left bond and the MPO left bond
    const QIndex& bond_in = left ? QL : QR;
    const QIndex& w_in = left ? W.legs[2] : W.legs[3];
    const QIndex& w_out = left ? W.legs[3] : W.legs[2];
    const QIndex& bond_out = left ? QR : QL;
    if (!env_ket.same_as(bond_in) || !env_mpo.same_as(w_in)) {
        err = left ? "left environment legs differ from the MPS left bond / MPO left bond"
                   : "right environment legs differ from the MPS right bond / MPO right bond";
        return TK_ERR_SECTOR_MISMATCH;
    }
    std::vector<double> Wd;
    if (!mpo_dense(W, Wd, err)) return TK_ERR_SECTOR_MISMATCH;
    const int64_t d = P.total, nwl = W.legs[2].total, nwr = W.legs[3].total;
    auto wval = [&](int64_t s, int64_t so, int64_t wl, int64_t wr) { return Wd[((s * d + so) * nwl + wl) * nwr + wr]; };
    std::vector<int> ssec;
    std::vector<int64_t> sloc;
    state_map(P, ssec, sloc);
    std::vector<int> win_sec, wout_sec;
    std::vector<int64_t> win_loc, wout_loc;
    state_map(w_in, win_sec, win_loc);
    state_map(w_out, wout_sec, wout_loc);
    EnvLayout lin, lout;
    env_layout(kind, bond_in, w_in, bond_in, lin);
    env_layout(kind, bond_out, w_out, bond_out, lout);
    G.out_total = lout.total;
    G.in_total = lin.total;
    const int nbi = bond_in.n(), nwi = w_in.n();
    std::vector<int64_t> in_blk((size_t)nbi * nwi * nbi, -1);
    for (size_t k = 0; k < lin.tri.size(); ++k)
        in_blk[((size_t)lin.tri[k][0] * nwi + lin.tri[k][1]) * nbi + lin.tri[k][2]] = lin.off[k];
    const int nl = QL.n();

    if (left) {
        // stage 1: T1(s, A', ws)[(a', w)][b] = L(A', ws, A)[(a', w)][a] * A(s, A, B)[a][b], A = A' - q(ws)
        std::map<std::array<int64_t, 3>, std::pair<int64_t, int>> t1;  // (s, A', ws) -> (offset, B)
        for (int64_t s = 0; s < d; ++s)
            for (int ap = 0; ap < nbi; ++ap)
                for (int ws = 0; ws < nwi; ++ws) {
                    Qn qa = qn_fuse(kind, QL.q[ap], qn_dual(kind, w_in.q[ws]));
                    int a = QL.find(qa);
                    if (a < 0) continue;
                    int64_t lo = in_blk[((size_t)ap * nwi + ws) * nbi + a];
                    int b = -1;
                    int64_t so = site_sub(A, ssec, sloc, s, a, &b);
                    if (lo < 0 || so < 0) continue;
                    GemmSeg sg{};
                    sg.a_off = lo; sg.a_rs = (int32_t)QL.dim[a]; sg.a_cs = 1;
                    sg.b_off = so; sg.b_rs = (int32_t)QR.dim[b]; sg.b_cs = 1;
                    sg.K = (int32_t)QL.dim[a];
                    GemmTask tk{};
                    tk.M = (int32_t)(QL.dim[ap] * w_in.dim[ws]);
                    tk.N = (int32_t)QR.dim[b];
                    tk.c_off = G.t1_total; tk.c_rs = tk.N; tk.c_cs = 1;
                    tk.seg_begin = (int)G.g1.segs.size();
                    G.g1.segs.push_back(sg);
                    tk.seg_end = (int)G.g1.segs.size();
                    tk.alpha = 1.0; tk.beta = 0.0;
                    G.g1.flops += 2.0 * tk.M * tk.N * (double)sg.K;
                    G.g1.tasks.push_back(tk);
                    gemm_add_tiles(G.g1, (int)G.g1.tasks.size() - 1, kEnvTileM, kEnvTileN);
                    t1[{s, ap, ws}] = {G.t1_total, b};
                    G.t1_total += (int64_t)tk.M * tk.N;
                }
        // stages 2 and 3, per output block (B', vs, B)
        std::map<std::array<int64_t, 4>, int64_t> t2;  // (s', A', vs, B) -> offset
        for (size_t k = 0; k < lout.tri.size(); ++k) {
            const int bp = lout.tri[k][0], vs = lout.tri[k][1], b = lout.tri[k][2];
            const int64_t dvs = w_out.dim[vs];
            GemmTask tk{};
            tk.M = (int32_t)QR.dim[bp];
            tk.N = (int32_t)(dvs * QR.dim[b]);
            tk.c_off = lout.off[k]; tk.c_rs = tk.N; tk.c_cs = 1;
            tk.seg_begin = (int)G.g3.segs.size();
            tk.alpha = 1.0; tk.beta = 0.0;
            for (int64_t sp = 0; sp < d; ++sp) {
                // bra block (s', A', B'): A' = B' - q(s')
                Qn qap = qn_fuse(kind, QR.q[bp], qn_dual(kind, P.q[ssec[sp]]));
                int ap = QL.find(qap);
                if (ap < 0) continue;
                int rb = -1;
                int64_t bo = site_sub(A, ssec, sloc, sp, ap, &rb);
                if (bo < 0 || rb != bp) continue;
                std::array<int64_t, 4> key{sp, ap, vs, b};
                auto it = t2.find(key);
                if (it == t2.end()) {
                    // T2(s', A', vs, B)[(a', v)][b] = sum_{s, w} W[s, s', w, v] T1(s, A', ws(w))[(a', w)][b]
                    const int64_t base = G.t2_total;
                    size_t job0 = G.jobs.size(), term0 = G.terms.size();
                    for (int64_t vl = 0; vl < dvs; ++vl) {
                        const int64_t v = w_out.off[vs] + vl;
                        CombJob j{};
                        j.rows = (int32_t)QL.dim[ap];
                        j.cols = (int32_t)QR.dim[b];
                        j.out_off = base + vl * QR.dim[b];
                        j.out_rs = (int32_t)(dvs * QR.dim[b]);
                        j.term_begin = (int32_t)G.terms.size();
                        for (int64_t s = 0; s < d; ++s)
                            for (int64_t w = 0; w < w_in.total; ++w) {
                                const double c = wval(s, sp, left ? w : v, left ? v : w);
                                if (c == 0.0) continue;
                                auto t = t1.find({s, ap, win_sec[w]});
                                if (t == t1.end() || t->second.second != b) continue;
                                CombTerm ct{};
                                ct.in_off = t->second.first + win_loc[w] * QR.dim[b];
                                ct.in_rs = (int32_t)(w_in.dim[win_sec[w]] * QR.dim[b]);
                                ct.coef = c;
                                G.terms.push_back(ct);
                                G.comb_flops += 2.0 * j.rows * j.cols;
                            }
                        j.term_end = (int32_t)G.terms.size();
                        G.jobs.push_back(j);
                    }
                    if (G.terms.size() == term0) {  // nothing reaches this block
                        G.jobs.resize(job0);
                        t2[key] = -1;
                        continue;
                    }
                    G.t2_total += QL.dim[ap] * dvs * QR.dim[b];
                    it = t2.emplace(key, base).first;
                }
                if (it->second < 0) continue;
                // L'(B', vs, B)[b'][(v, b)] += A(s', A', B')^T[b'][a'] * T2[a'][(v, b)]
                GemmSeg sg{};
                sg.a_off = bo; sg.a_rs = 1; sg.a_cs = (int32_t)QR.dim[bp];
                sg.b_off = it->second; sg.b_rs = tk.N; sg.b_cs = 1;
                sg.K = (int32_t)QL.dim[ap];
                G.g3.segs.push_back(sg);
                G.g3.flops += 2.0 * tk.M * tk.N * (double)sg.K;
            }
            tk.seg_end = (int)G.g3.segs.size();
            if (tk.seg_end == tk.seg_begin) continue;  // stays zero
            G.g3.tasks.push_back(tk);
            gemm_add_tiles(G.g3, (int)G.g3.tasks.size() - 1, kEnvTileM, kEnvTileN);
        }
    } else {
        // stage 1: T1(s, A, v)[a][b'] = A(s, A, B)[a][b] * R(B', vs, B)[b'][v][b], B' = B + q(vs)
        std::map<std::array<int64_t, 3>, std::pair<int64_t, int>> t1;  // (s, A, v) -> (offset, B')
        for (int64_t s = 0; s < d; ++s)
            for (int a = 0; a < nl; ++a) {
                int b = -1;
                int64_t so = site_sub(A, ssec, sloc, s, a, &b);
                if (so < 0) continue;
                for (int vs = 0; vs < nwi; ++vs) {
                    int bp = QR.find(qn_fuse(kind, QR.q[b], w_in.q[vs]));
                    if (bp < 0) continue;
                    int64_t ro = in_blk[((size_t)bp * nwi + vs) * nbi + b];
                    if (ro < 0) continue;
                    for (int64_t vl = 0; vl < w_in.dim[vs]; ++vl) {
                        GemmSeg sg{};
                        sg.a_off = so; sg.a_rs = (int32_t)QR.dim[b]; sg.a_cs = 1;
                        sg.b_off = ro + vl * QR.dim[b]; sg.b_rs = 1; sg.b_cs = (int32_t)(w_in.dim[vs] * QR.dim[b]);
                        sg.K = (int32_t)QR.dim[b];
                        GemmTask tk{};
                        tk.M = (int32_t)QL.dim[a];
                        tk.N = (int32_t)QR.dim[bp];
                        tk.c_off = G.t1_total; tk.c_rs = tk.N; tk.c_cs = 1;
                        tk.seg_begin = (int)G.g1.segs.size();
                        G.g1.segs.push_back(sg);
                        tk.seg_end = (int)G.g1.segs.size();
                        tk.alpha = 1.0; tk.beta = 0.0;
                        G.g1.flops += 2.0 * tk.M * tk.N * (double)sg.K;
                        G.g1.tasks.push_back(tk);
                        gemm_add_tiles(G.g1, (int)G.g1.tasks.size() - 1, kEnvTileM, kEnvTileN);
                        t1[{s, a, w_in.off[vs] + vl}] = {G.t1_total, bp};
                        G.t1_total += (int64_t)tk.M * tk.N;
                    }
                }
            }
        // stages 2 and 3, per output block (A', ws, A) and channel state w
        std::map<std::array<int64_t, 4>, int64_t> t2;  // (s', A, w, B') -> offset
        for (size_t k = 0; k < lout.tri.size(); ++k) {
            const int ap = lout.tri[k][0], ws = lout.tri[k][1], a = lout.tri[k][2];
            const int64_t dws = w_out.dim[ws];
            for (int64_t wl = 0; wl < dws; ++wl) {
                const int64_t w = w_out.off[ws] + wl;
                GemmTask tk{};
                tk.M = (int32_t)QL.dim[ap];
                tk.N = (int32_t)QL.dim[a];
                tk.c_off = lout.off[k] + wl * QL.dim[a]; tk.c_rs = (int32_t)(dws * QL.dim[a]); tk.c_cs = 1;
                tk.seg_begin = (int)G.g3.segs.size();
                tk.alpha = 1.0; tk.beta = 0.0;
                for (int64_t sp = 0; sp < d; ++sp) {
                    int bp = -1;
                    int64_t bo = site_sub(A, ssec, sloc, sp, ap, &bp);  // bra block (s', A', B')
                    if (bo < 0) continue;
                    std::array<int64_t, 4> key{sp, a, w, bp};
                    auto it = t2.find(key);
                    if (it == t2.end()) {
                        // T2(s', A, w, B')[a][b'] = sum_{s, v} W[s, s', w, v] T1(s, A, v)[a][b']
                        CombJob j{};
                        j.rows = (int32_t)QL.dim[a];
                        j.cols = (int32_t)QR.dim[bp];
                        j.out_off = G.t2_total;
                        j.out_rs = j.cols;
                        j.term_begin = (int32_t)G.terms.size();
                        for (int64_t s = 0; s < d; ++s)
                            for (int64_t v = 0; v < w_in.total; ++v) {
                                const double c = wval(s, sp, w, v);
                                if (c == 0.0) continue;
                                auto t = t1.find({s, a, v});
                                if (t == t1.end() || t->second.second != bp) continue;
                                CombTerm ct{};
                                ct.in_off = t->second.first;
                                ct.in_rs = j.cols;
                                ct.coef = c;
                                G.terms.push_back(ct);
                                G.comb_flops += 2.0 * j.rows * j.cols;
                            }
                        j.term_end = (int32_t)G.terms.size();
                        if (j.term_end == j.term_begin) {
                            t2[key] = -1;
                            continue;
                        }
                        G.jobs.push_back(j);
                        it = t2.emplace(key, G.t2_total).first;
                        G.t2_total += (int64_t)j.rows * j.cols;
                    }
                    if (it->second < 0) continue;
                    // R'(A', ws, A)[a'][(w, a)] += A(s', A', B')[a'][b'] * T2[a][b']^T
                    GemmSeg sg{};
                    sg.a_off = bo; sg.a_rs = (int32_t)QR.dim[bp]; sg.a_cs = 1;
                    sg.b_off = it->second; sg.b_rs = 1; sg.b_cs = (int32_t)QR.dim[bp];
                    sg.K = (int32_t)QR.dim[bp];
                    G.g3.segs.push_back(sg);
                    G.g3.flops += 2.0 * tk.M * tk.N * (double)sg.K;
                }
                tk.seg_end = (int)G.g3.segs.size();
                if (tk.seg_end == tk.seg_begin) continue;
                G.g3.tasks.push_back(tk);
                gemm_add_tiles(G.g3, (int)G.g3.tasks.size() - 1, kEnvTileM, kEnvTileN);
            }
        }
    }
    if (!finish(G, lin.total, A.total, lout.total, left, err)) return TK_ERR_INVALID_ARG;
    return TK_OK;
}

tk_status build_grow_tables(bool left, const QIndex& env_bra, const QIndex& env_mpo, const QIndex& env_ket,
                            const Bst3& A, const Bst4& W, GrowTables& G, std::string& err) {
    return guard_host("environment growth tables", err,
                      [&] { return build_grow_tables_body(left, env_bra, env_mpo, env_ket, A, W, G, err); });
}

static tk_status build_product_tables_body(const Heff2Tables& H, const Bst3& Ai, const Bst3& Aj, GemmTable& g,
                                           std::string& err) {
    g = GemmTable();
    const int kind = Ai.kind;
    const QIndex& PI = Ai.legs[0];
    const QIndex& QA = Ai.legs[1];
    const QIndex& QC = Ai.legs[2];
    const QIndex& PJ = Aj.legs[0];
    const QIndex& QB = Aj.legs[2];
    if (!QC.same_as(Aj.legs[1])) {
        err = "A_i right bond and A_j left bond QIndex differ";
        return TK_ERR_SECTOR_MISMATCH;
    }
    if (PI.total != H.d_i || PJ.total != H.d_j || QA.total != H.d_l || QB.total != H.d_r || kind != H.kind) {
        err = "MPS site legs differ from the plan's two-site legs";
        return TK_ERR_SECTOR_MISMATCH;
    }
    for (size_t k = 0; k < H.keys.size(); ++k) {
        Qn q[4];
        key_unpack(kind, H.keys[k], 4, q);
        int si = PI.find(q[0]), sj = PJ.find(q[1]), a = QA.find(q[2]), b = QB.find(q[3]);
        if (si < 0 || sj < 0 || a < 0 || b < 0) {
            err = "plan block names a sector missing from the MPS legs";
            return TK_ERR_SECTOR_MISMATCH;
        }
        const int c = QC.find(qn_fuse(kind, q[0], q[2]));
        const int64_t ni = PI.dim[si], nj = PJ.dim[sj], DA = QA.dim[a], DB = QB.dim[b];
        for (int64_t li = 0; li < ni; ++li)
            for (int64_t lj = 0; lj < nj; ++lj) {
                if (c < 0) continue;
                const int64_t bi = Ai.blk[(size_t)si * QA.n() + a];
                const int64_t bj = Aj.blk[(size_t)sj * QC.n() + c];
                if (bi < 0 || bj < 0 || Aj.right[(size_t)sj * QC.n() + c] != b) continue;
                const int64_t DC = QC.dim[c];
                GemmSeg sg{};
                sg.a_off = bi + li * DA * DC; sg.a_rs = (int32_t)DC; sg.a_cs = 1;
                sg.b_off = bj + lj * DC * DB; sg.b_rs = (int32_t)DB; sg.b_cs = 1;
                sg.K = (int32_t)DC;
                GemmTask tk{};
                tk.M = (int32_t)DA;
                tk.N = (int32_t)DB;
                tk.c_off = H.blk_off[k] + (li * nj + lj) * DA * DB; tk.c_rs = tk.N; tk.c_cs = 1;
                tk.seg_begin = (int)g.segs.size();
                g.segs.push_back(sg);
                tk.seg_end = (int)g.segs.size();
                tk.alpha = 1.0; tk.beta = 0.0;
                g.flops += 2.0 * tk.M * tk.N * (double)sg.K;
                g.tasks.push_back(tk);
                gemm_add_tiles(g, (int)g.tasks.size() - 1, kEnvTileM, kEnvTileN);
            }
    }
    gemm_lpt_order(g, kEnvTileM, kEnvTileN);
    if (!gemm_table_ok(g, Ai.total, Aj.total, H.total, "two-site product", err)) return TK_ERR_INVALID_ARG;
    return TK_OK;
}

tk_status build_product_tables(const Heff2Tables& H, const Bst3& Ai, const Bst3& Aj, GemmTable& g, std::string& err) {
    return guard_host("two-site product tables", err, [&] { return build_product_tables_body(H, Ai, Aj, g, err); });
}

}  // namespace tk
