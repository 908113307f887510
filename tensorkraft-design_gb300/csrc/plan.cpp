// plan.cpp -- host-side sector bookkeeping for the two-site H_eff.
//
// Integer work only: decodes the reference-format inputs (dense
// environments, block-sparse MPO tensors), enumerates the two-site sectors,
// finds the non-zero environment slabs and flattens every sector GEMM of one
// matvec into task tables that the device kernels walk.
//
// Reference semantics followed (kyungminlee/tensorkraft-design):
//   tk-dmrg/src/environments/mod.rs:491-602  which (L, W_i, W_j, R) entries meet
//       which (in, out) pair: in=(s_i,s_j,a_L,a_R), out=(s'_i,s'_j,a'_L,a'_R),
//       L(a'_L, w_L, a_L), R(a'_R, w_R, a_R), w_mid paired by quantum number
//       with the block-local index (:532, :545), physical and MPO-bond offsets
//       from the MPO's QIndex order (:518-538).
//   tk-symmetry/src/flux.rs:43-234  sector enumeration (DFS order, last leg solved).
//   tk-symmetry/src/block_sparse.rs:40-84  blocks sorted by packed key.
//   tk-symmetry/src/flat_storage.rs:95-130  blocks back to back, row-major.
//   tk-linalg/src/tasks.rs:172-174  LPT order (heaviest work first).
#include <algorithm>
#include <array>
#include <climits>
#include <cmath>
#include <cstring>
#include <atomic>
#include <memory>
#include <numeric>
#include <system_error>
#include <thread>
#include <unordered_map>

#include "tk_internal.hpp"

namespace tk {

static std::atomic<int> g_fail_host_alloc{0};

void host_alloc_checkpoint() {
    int c = g_fail_host_alloc.load(std::memory_order_relaxed);
    while (c > 0 && !g_fail_host_alloc.compare_exchange_weak(c, c - 1)) {
    }
    if (c == 1) throw std::bad_alloc();
}

int qn_ncomp(int kind) { return (kind == TK_QN_U1Z2 || kind == TK_QN_U1U1) ? 2 : 1; }

int qn_bits(int kind) {
    switch (kind) {
    case TK_QN_U1: return 8;
    case TK_QN_Z2: return 1;
    case TK_QN_U1Z2: return 9;
    case TK_QN_U1WIDE: return 16;
    case TK_QN_U1U1: return 16;
    default: return -1;
    }
}

bool qn_kind_valid(int kind) { return qn_bits(kind) > 0; }

Qn qn_fuse(int kind, const Qn& a, const Qn& b) {
    Qn r;
    switch (kind) {
    case TK_QN_Z2: r.c[0] = a.c[0] ^ b.c[0]; break;
    case TK_QN_U1Z2: r.c[0] = a.c[0] + b.c[0]; r.c[1] = a.c[1] ^ b.c[1]; break;
    case TK_QN_U1U1: r.c[0] = a.c[0] + b.c[0]; r.c[1] = a.c[1] + b.c[1]; break;
    default: r.c[0] = a.c[0] + b.c[0]; break;
    }
    return r;
}

Qn qn_dual(int kind, const Qn& a) {
    Qn r;
    switch (kind) {
    case TK_QN_Z2: r.c[0] = a.c[0]; break;
    case TK_QN_U1Z2: r.c[0] = -a.c[0]; r.c[1] = a.c[1]; break;
    case TK_QN_U1U1: r.c[0] = -a.c[0]; r.c[1] = -a.c[1]; break;
    default: r.c[0] = -a.c[0]; break;
    }
    return r;
}

bool qn_less(const Qn& a, const Qn& b) {
    if (a.c[0] != b.c[0]) return a.c[0] < b.c[0];
    return a.c[1] < b.c[1];
}

static int32_t low_signed(uint64_t v, int bits) {
    uint64_t m = (1ull << bits) - 1;
    v &= m;
    return (v >> (bits - 1)) ? (int32_t)((int64_t)v - (int64_t)(1ull << bits)) : (int32_t)v;
}

uint64_t qn_pack(int kind, const Qn& q) {
    switch (kind) {
    case TK_QN_U1: return (uint64_t)((uint32_t)q.c[0] & 0xFFu);
    case TK_QN_Z2: return (uint64_t)(q.c[0] != 0);
    case TK_QN_U1Z2: return (uint64_t)((uint32_t)q.c[0] & 0xFFu) | ((uint64_t)(q.c[1] != 0) << 8);
    case TK_QN_U1WIDE: return (uint64_t)((uint32_t)q.c[0] & 0xFFFFu);
    case TK_QN_U1U1: return (uint64_t)((uint32_t)q.c[0] & 0xFFu) | ((uint64_t)((uint32_t)q.c[1] & 0xFFu) << 8);
    default: return 0;
    }
}

Qn qn_unpack(int kind, uint64_t b) {
    Qn q;
    switch (kind) {
    case TK_QN_U1: q.c[0] = low_signed(b, 8); break;
    case TK_QN_Z2: q.c[0] = (int32_t)(b & 1); break;
    case TK_QN_U1Z2: q.c[0] = low_signed(b, 8); q.c[1] = (int32_t)((b >> 8) & 1); break;
    case TK_QN_U1WIDE: q.c[0] = low_signed(b, 16); break;
    case TK_QN_U1U1: q.c[0] = low_signed(b, 8); q.c[1] = low_signed(b >> 8, 8); break;
    default: break;
    }
    return q;
}

uint64_t key_pack(int kind, const Qn* qns, int rank) {
    int bw = qn_bits(kind);
    uint64_t mask = (bw >= 64) ? ~0ull : ((1ull << bw) - 1);
    uint64_t key = 0;
    for (int i = 0; i < rank; ++i) key |= (qn_pack(kind, qns[i]) & mask) << (i * bw);
    return key;
}

void key_unpack(int kind, uint64_t key, int rank, Qn* qns) {
    int bw = qn_bits(kind);
    uint64_t mask = (1ull << bw) - 1;
    for (int i = 0; i < rank; ++i) qns[i] = qn_unpack(kind, (key >> (i * bw)) & mask);
}

uint16_t f32_to_bf16_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

float bf16_bits_to_f32(uint16_t b) {
    uint32_t u = (uint32_t)b << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

int QIndex::find(const Qn& x) const {
    for (size_t s = 0; s < q.size(); ++s)
        if (q[s] == x) return (int)s;
    return -1;
}

bool QIndex::same_as(const QIndex& o) const {
    if (q.size() != o.q.size()) return false;
    for (size_t s = 0; s < q.size(); ++s)
        if (q[s] != o.q[s] || dim[s] != o.dim[s]) return false;
    return true;
}

bool qindex_from_abi(int kind, const tk_qindex& in, QIndex& out, std::string& err) {
    int nc = qn_ncomp(kind);
    if (in.n_sectors < 0 || (in.n_sectors > 0 && (!in.charges || !in.dims))) {
        err = "QIndex: null charges/dims";
        return false;
    }
    out.q.resize(in.n_sectors);
    out.dim.resize(in.n_sectors);
    out.off.resize(in.n_sectors);
    out.total = 0;
    for (int s = 0; s < in.n_sectors; ++s) {
        Qn q;
        for (int k = 0; k < nc; ++k) q.c[k] = in.charges[s * nc + k];
        out.q[s] = q;
        if (in.dims[s] <= 0) {
            err = "QIndex: sector with non-positive dimension";
            return false;
        }
        out.dim[s] = in.dims[s];
        out.off[s] = out.total;
        out.total += in.dims[s];
        if (s > 0 && !qn_less(out.q[s - 1], q)) {
            err = "QIndex: sectors not strictly sorted by quantum number";
            return false;
        }
    }
    return true;
}

bool bst4_from_abi(const tk_bst& t, Bst4& o, const char* name, std::string& err) {
    if (t.rank != 4 || !t.legs) {
        err = std::string(name) + ": MPO site tensor must have rank 4 (s_in, s_out, w_L, w_R)";
        return false;
    }
    if (!qn_kind_valid(t.qn_kind)) {
        err = std::string(name) + ": unknown quantum-number kind";
        return false;
    }
    o.kind = t.qn_kind;
    for (int l = 0; l < 4; ++l)
        if (!qindex_from_abi(t.qn_kind, t.legs[l], o.legs[l], err)) {
            err = std::string(name) + ": " + err;
            return false;
        }
    if (t.n_blocks < 0 || (t.n_blocks > 0 && (!t.keys || !t.block_offsets || !t.data))) {
        err = std::string(name) + ": null block arrays";
        return false;
    }
    o.keys.assign(t.keys, t.keys + t.n_blocks);
    o.offs.assign(t.block_offsets, t.block_offsets + t.n_blocks);
    o.data = t.data;
    for (int64_t b = 1; b < t.n_blocks; ++b)
        if (o.keys[b - 1] >= o.keys[b]) {
            err = std::string(name) + ": sector keys not strictly ascending";
            return false;
        }
    return true;
}

// Dense MPO tensor (d, d, wl, wr) in global indices, following the offsets
// the reference reads (environments/mod.rs:518-538, `unwrap_or(0)` for absent
// sectors is an error here).
bool mpo_dense(const Bst4& w, std::vector<double>& out, std::string& err) {
    int64_t d0 = w.legs[0].total, d1 = w.legs[1].total, d2 = w.legs[2].total, d3 = w.legs[3].total;
    out.assign((size_t)(d0 * d1 * d2 * d3), 0.0);
    for (size_t b = 0; b < w.keys.size(); ++b) {
        Qn q[4];
        key_unpack(w.kind, w.keys[b], 4, q);
        int s[4];
        for (int l = 0; l < 4; ++l) {
            s[l] = w.legs[l].find(q[l]);
            if (s[l] < 0) {
                err = "MPO block key names a sector missing from its QIndex";
                return false;
            }
        }
        int64_t n0 = w.legs[0].dim[s[0]], n1 = w.legs[1].dim[s[1]], n2 = w.legs[2].dim[s[2]], n3 = w.legs[3].dim[s[3]];
        const double* blk = w.data + w.offs[b];
        for (int64_t i0 = 0; i0 < n0; ++i0)
            for (int64_t i1 = 0; i1 < n1; ++i1)
                for (int64_t i2 = 0; i2 < n2; ++i2)
                    for (int64_t i3 = 0; i3 < n3; ++i3) {
                        int64_t g0 = w.legs[0].off[s[0]] + i0, g1 = w.legs[1].off[s[1]] + i1;
                        int64_t g2 = w.legs[2].off[s[2]] + i2, g3 = w.legs[3].off[s[3]] + i3;
                        out[((g0 * d1 + g1) * d2 + g2) * d3 + g3] += blk[((i0 * n1 + i1) * n2 + i2) * n3 + i3];
                    }
    }
    return true;
}

namespace {

// enumerate_valid_sectors (flux.rs:43-234) for the two-site tensor, directions
// (In, In, In, Out): q(s_i) + q(s_j) + q(a_L) - q(a_R) == flux.
void enumerate4(int kind, const QIndex* legs, const Qn& flux, std::vector<std::array<int, 4>>& out) {
    for (int a = 0; a < legs[0].n(); ++a)
        for (int b = 0; b < legs[1].n(); ++b)
            for (int c = 0; c < legs[2].n(); ++c) {
                Qn part = qn_fuse(kind, qn_fuse(kind, legs[0].q[a], legs[1].q[b]), legs[2].q[c]);
                // Outgoing last leg: required = dual(flux (+) dual(partial)) = partial (+) dual(flux)
                Qn req = qn_dual(kind, qn_fuse(kind, flux, qn_dual(kind, part)));
                int d = legs[3].find(req);
                if (d >= 0) out.push_back({a, b, c, d});
            }
}

}  // namespace

static void add_tiles(GemmTable& g, int task_id, int tile_m, int tile_n, const std::vector<int64_t>&) {
    gemm_add_tiles(g, task_id, tile_m, tile_n);
}

int gemm_tile_class(int M, int N) {
    // square tiles of edge 64 >> cls; cost = tiles x (area + a fixed per-tile share)
    int best = 0;
    double best_cost = 0.0;
    for (int cls = 0; cls < kGemmTileClasses; ++cls) {
        const int e = 64 >> cls;
        const double cost = (double)((M + e - 1) / e) * ((N + e - 1) / e) * ((double)e * e + 256.0);
        if (cls == 0 || cost < best_cost) {
            best = cls;
            best_cost = cost;
        }
    }
    return best;
}

void gemm_add_tiles(GemmTable& g, int task_id, int tile_m, int tile_n) {
    const GemmTask& t = g.tasks[task_id];
    const int cls = (tile_m == 64 && tile_n == 64) ? gemm_tile_class(t.M, t.N) : 0;
    const int e = 64 >> cls;
    for (int m0 = 0; m0 < t.M; m0 += e)
        for (int n0 = 0; n0 < t.N; n0 += e) g.tiles.push_back({task_id, m0, n0, cls});
}

static void lpt_order(GemmTable& g, int tile_m, int tile_n) { gemm_lpt_order(g, tile_m, tile_n); }

void gemm_lpt_order(GemmTable& g, int tile_m, int tile_n) {
    // Cost of a tile = (rows) x (cols) x (total K); heaviest first.
    std::vector<double> ktot(g.tasks.size(), 0.0);
    for (size_t t = 0; t < g.tasks.size(); ++t)
        for (int s = g.tasks[t].seg_begin; s < g.tasks[t].seg_end; ++s) ktot[t] += g.segs[s].K;
    auto cost = [&](const GemmTile& x) {
        const GemmTask& t = g.tasks[x.task];
        const int e = std::min(tile_m, 64 >> x.cls);
        double rm = std::min(e, t.M - x.m0), rn = std::min(std::min(tile_n, 64 >> x.cls), t.N - x.n0);
        return (ktot[x.task] + 1.0) * rm * rn;
    };
    std::stable_sort(g.tiles.begin(), g.tiles.end(),
                     [&](const GemmTile& a, const GemmTile& b) { return cost(a) > cost(b); });
}

// Every device access the tables can produce, checked against its buffer on
// the host: a table fault becomes an error code instead of a device fault.
bool gemm_table_ok(const GemmTable& g, int64_t na, int64_t nb, int64_t nc, const char* name, std::string& err) {
        for (const GemmTile& tl : g.tiles) {
            if (tl.task < 0 || (size_t)tl.task >= g.tasks.size()) { err = std::string(name) + ": tile task"; return false; }
            if (tl.cls < 0 || tl.cls >= kGemmTileClasses) { err = std::string(name) + ": tile class"; return false; }
            const GemmTask& t = g.tasks[tl.task];
            if (tl.m0 < 0 || tl.m0 >= t.M || tl.n0 < 0 || tl.n0 >= t.N) { err = std::string(name) + ": tile origin"; return false; }
        }
        for (const GemmTask& t : g.tasks) {
            if (t.M <= 0 || t.N <= 0) { err = std::string(name) + ": empty task"; return false; }
            int64_t cmax = t.c_off + (int64_t)(t.M - 1) * t.c_rs + (int64_t)(t.N - 1) * t.c_cs;
            if (t.c_off < 0 || cmax >= nc) { err = std::string(name) + ": output range"; return false; }
            if (t.seg_begin < 0 || t.seg_end < t.seg_begin || (size_t)t.seg_end > g.segs.size()) { err = std::string(name) + ": segments"; return false; }
            for (int s = t.seg_begin; s < t.seg_end; ++s) {
                const GemmSeg& sg = g.segs[s];
                int64_t amax = sg.a_off + (int64_t)(t.M - 1) * sg.a_rs + (int64_t)(sg.K - 1) * sg.a_cs;
                int64_t bmax = sg.b_off + (int64_t)(sg.K - 1) * sg.b_rs + (int64_t)(t.N - 1) * sg.b_cs;
                if (sg.K <= 0 || sg.a_off < 0 || sg.b_off < 0 || amax >= na || bmax >= nb) { err = std::string(name) + ": operand range"; return false; }
            }
        }
        return true;
}

bool comb_table_ok(const std::vector<CombJob>& jobs, const std::vector<CombTerm>& terms, int64_t n_in, int64_t n_out,
                   std::string& err) {
    for (const CombJob& j : jobs) {
        if (j.rows <= 0 || j.cols <= 0 || j.out_off < 0 || j.out_off + (int64_t)(j.rows - 1) * j.out_rs + j.cols - 1 >= n_out ||
            j.term_begin < 0 || j.term_end < j.term_begin || (size_t)j.term_end > terms.size()) { err = "combine job range"; return false; }
        for (int t = j.term_begin; t < j.term_end; ++t) {
            const CombTerm& c = terms[t];
            if (c.in_off < 0 || c.in_off + (int64_t)(j.rows - 1) * c.in_rs + j.cols - 1 >= n_in) { err = "combine term range"; return false; }
        }
    }
    return true;
}

static bool validate_tc(const Heff2Tables& T, const TcTables& C, std::string& err);

static bool validate_tables(const Heff2Tables& T, std::string& err) {
    if (!gemm_table_ok(T.g1, (int64_t)T.lbuf.size(), T.total, T.t1_total, "stage 1", err)) return false;
    if (!gemm_table_ok(T.g3, T.t2_total, (int64_t)T.rbuf.size(), T.total, "stage 3", err)) return false;
    if (!comb_table_ok(T.jobs, T.terms, T.t1_total, T.t2_total, err)) return false;
    return !T.tc_built || validate_tc(T, T.tc, err);
}

// Every access of the split (or stacked FP64) tables checked against its buffer.
static bool validate_tc(const Heff2Tables& T, const TcTables& C, std::string& err) {
    if (!C.term_coef64.empty() && C.term_coef64.size() != C.terms.size()) {
        err = "FP64 combine coefficients";
        return false;
    }
    // operand stacks: the last row a tile reads (TMA reads past the end
    // would be zero-filled; the stacked FP64 kernels read them directly)
    auto last_row = [](int32_t row, int32_t cs, int32_t kch, int32_t valid) {
        return (int64_t)row + (int64_t)std::max(kch - 1, 0) * cs + valid - 1;
    };
    for (const TcTile& t : C.tiles3)
        if (t.k_valid < 0 || t.k_valid > t.kch * kTcBK || t.a_cs < 0 || t.b_cs < 0 ||
            (t.kch > 0 && (last_row(t.a_row, t.a_cs, t.kch, t.m_valid) >= C.t2q_rows ||
                           last_row(t.b_row, t.b_cs, t.kch, t.n_valid) >= C.rq_rows))) {
            err = "tensor-core stage 3 operand";
            return false;
        }
    for (const std::vector<TcTile>* v : {&C.tiles1, &C.tiles1x})
        for (const TcTile& t : *v)
            if (t.a_cs < 0 || (t.kch > 0 && last_row(t.a_row, t.a_cs, t.kch, t.m_valid) >= C.lq_rows)) {
                err = "tensor-core stage 1 operand";
                return false;
            }
    if (C.t1col_base.size() != C.t1col_stride.size() || C.xsrc.size() != C.t1col_base.size() ||
        C.xstride.size() != C.t1col_base.size()) {
        err = "T1 column tables";
        return false;
    }
    for (const TcTile& t : C.tiles1x) {
        if (t.b_cs <= 0 || t.kch <= 0 ||
            (int64_t)t.b_row + (int64_t)(t.kch - 1) * t.b_cs + t.n_valid - 1 >= C.xq_rows) {
            err = "tensor-core stage 1 split-copy operand";
            return false;
        }
    }
    for (const TcSplitJob& j : C.split) {
        const int64_t nb = std::min<int64_t>(32, (int64_t)j.cols - j.b0);
        const int64_t imax = (((int64_t)j.xrow + (int64_t)(j.a0 / kTcBK) * j.cstride + j.b0 + nb - 1) << 6) + 63;
        if (j.rows <= 0 || j.cols <= 0 || j.src < 0 || j.src + (int64_t)j.rows * j.cols > T.total || j.xrow < 0 ||
            j.cstride <= 0 || j.a0 < 0 || j.a0 >= j.rows || j.a0 % kTcBK != 0 || j.b0 < 0 || j.b0 >= j.cols ||
            imax >= C.xq_rows * kTcBK) {
            err = "tensor-core split job";
            return false;
        }
    }
    auto tile1_ok = [&](const TcTile& t) {
        if (t.mode != 2 || t.m_valid <= 0 || t.n_valid <= 0 || t.m_valid > kTcBM || t.n_valid > kTcBN || t.kch < 0 ||
            t.n_mma < t.n_valid || t.n_mma > kTcBN || t.n_mma % 16 != 0 || t.out_off < 0 || t.ldc < 0 ||
            t.out_off + t.n_valid > (int64_t)C.t1col_base.size() || t.a_row < 0 || t.b_row < 0) {
            err = "tensor-core stage 1 tile";
            return false;
        }
        if (t.k_valid <= 0 || t.k_valid > t.kch * kTcBK || t.k_valid <= (t.kch - 1) * kTcBK) {
            err = "tensor-core stage 1 K";
            return false;
        }
        for (int c = 0; c < t.n_valid; ++c) {
            const int64_t base = C.t1col_base[t.out_off + c], st = C.t1col_stride[t.out_off + c];
            if (base < 0 || st <= 0 || base + (int64_t)(t.ldc + t.m_valid - 1) * st >= C.t1_total) {
                err = "tensor-core stage 1 output column";
                return false;
            }
            const int64_t xs = C.xsrc[t.out_off + c], xst = C.xstride[t.out_off + c];
            if (xs < 0 || xst <= 0 || xs + (int64_t)(t.k_valid - 1) * xst >= T.total) {
                err = "tensor-core stage 1 psi column";
                return false;
            }
        }
        return true;
    };
    for (const TcTile& t : C.tiles1)
        if (!tile1_ok(t)) return false;
    if (C.x_cut[0] != 0 || C.x_cut[kTcPsiPieces] != T.total || C.n1_cut[0] != 0 ||
        C.n1_cut[kTcPsiPieces] != (int32_t)C.tiles1.size()) {
        err = "tensor-core stage 1 psi pieces";
        return false;
    }
    for (int j = 0; j < kTcPsiPieces; ++j) {
        if (C.x_cut[j + 1] < C.x_cut[j] || C.n1_cut[j + 1] < C.n1_cut[j]) {
            err = "tensor-core stage 1 psi pieces";
            return false;
        }
        for (int32_t i = C.n1_cut[j]; i < C.n1_cut[j + 1]; ++i) {
            const TcTile& t = C.tiles1[(size_t)i];
            for (int c = 0; c < t.n_valid; ++c)
                if (C.xsrc[t.out_off + c] + (int64_t)(t.k_valid - 1) * C.xstride[t.out_off + c] >= C.x_cut[j + 1]) {
                    err = "tensor-core stage 1 tile reads past its psi piece";
                    return false;
                }
        }
    }
    for (const TcTile& t : C.tiles1x)
        if (!tile1_ok(t)) return false;
    for (const TcTile& t : C.tiles3) {
        if (t.n_mma < t.n_valid || t.n_mma > kTcBN || t.n_mma % 16 != 0) { err = "tensor-core stage 3 tile N"; return false; }
        if (t.mode != 1 || t.m_valid <= 0 || t.n_valid <= 0 || t.m_valid > kTcBM || t.n_valid > kTcBN || t.kch < 0 ||
            t.out_off < 0 || t.out_off + t.m_valid - 1 >= (int64_t)C.yrow.size() || t.a_row < 0 || t.b_row < 0) {
            err = "tensor-core stage 3 tile";
            return false;
        }
        for (int r = 0; r < t.m_valid; ++r) {
            int64_t y0 = C.yrow[t.out_off + r];
            if (y0 < 0 || y0 + t.n0 + t.n_valid - 1 >= T.total) { err = "tensor-core stage 3 output row"; return false; }
        }
    }
    for (const TcTile& t : C.tiles3f) {
        if (t.mode != 3 || t.n_mma < t.n_valid || t.n_mma > kTcBN || t.n_mma % 16 != 0 || t.m_valid <= 0 ||
            t.n_valid <= 0 || t.m_valid > kTcBM || t.n_valid > kTcBN || t.kch < 0 || t.out_off < 0 ||
            t.out_off + t.m_valid - 1 >= (int64_t)C.yrow.size() || t.b_row < 0 || t.fill0 < 0 ||
            (size_t)t.fill0 + t.kch >= C.fill_chunk.size()) {
            err = "tensor-core fused stage 3 tile";
            return false;
        }
        for (int r = 0; r < t.m_valid; ++r) {
            int64_t y0 = C.yrow[t.out_off + r];
            if (y0 < 0 || y0 + t.n0 + t.n_valid - 1 >= T.total) { err = "tensor-core stage 3 output row"; return false; }
        }
        for (int c = 0; c < t.kch; ++c) {
            const int32_t a = C.fill_chunk[(size_t)t.fill0 + c], b = C.fill_chunk[(size_t)t.fill0 + c + 1];
            if (a < 0 || b < a || (size_t)b > C.fill_segs.size()) { err = "tensor-core fill chunk"; return false; }
        }
    }
    for (const TcFillSeg& g : C.fill_segs) {
        if (g.r0 < 0 || g.rows <= 0 || g.r0 + g.rows > kTcBM || g.k0 < 0 || g.cols <= 0 || g.k0 + g.cols > kTcBK ||
            g.term_begin < 0 || g.term_end < g.term_begin || (size_t)g.term_end > C.fill_terms.size()) {
            err = "tensor-core fill segment";
            return false;
        }
        for (int32_t t = g.term_begin; t < g.term_end; ++t) {
            const TcCombTerm& c = C.fill_terms[t];
            if (c.in_off < 0 || c.in_rs < 0 || c.in_off + (int64_t)(g.rows - 1) * c.in_rs + g.cols - 1 >= C.t1_total) {
                err = "tensor-core fill term";
                return false;
            }
        }
    }
    for (const TcCombJob& j : C.jobs) {
        int64_t kmax = (int64_t)j.k0 + j.cols - 1;
        int64_t imax = (((int64_t)j.t2row + (kmax >> 6) * j.cstride + j.r0 + j.rows - 1) << 6) + 63;
        if (j.rows <= 0 || j.cols <= 0 || j.r0 < 0 || (int64_t)j.rows * j.cols > kTcCombMaxElems + j.cols || j.k0 < 0 ||
            j.t2row < 0 || imax >= C.t2q_rows * kTcBK || j.term_begin < 0 || j.term_end < j.term_begin ||
            (size_t)j.term_end > C.terms.size()) { err = "tensor-core combine job"; return false; }
        for (int t = j.term_begin; t < j.term_end; ++t) {
            const TcCombTerm& c = C.terms[t];
            if (t - j.term_begin < kTcCombInline) {
                const TcCombTerm& d = j.inl[t - j.term_begin];
                if (d.in_off != c.in_off || d.in_rs != c.in_rs || d.coef != c.coef) {
                    err = "tensor-core combine inline term";
                    return false;
                }
            }
            if (c.in_off < 0 || c.in_off + (int64_t)(j.r0 + j.rows - 1) * c.in_rs + j.cols - 1 >= C.t1_total) {
                err = "tensor-core combine term";
                return false;
            }
        }
    }
    return true;
}

// One environment slab copied into a tensor-core operand stack: element
// (r, kk) of the row-major [nr x len] slab is column k of the stack's row r,
// k = k_off + kk, stored K-major in 64-wide chunks (chunk k / kTcBK holds
// chunk_rows rows starting at row0 + (k / kTcBK) * chunk_rows).
struct StackCopy {
    const double* src;
    int64_t nr, len, k_off, row0, chunk_rows;
};

// Every element of the stack copies, (destination index, value), to `put`,
// on up to 16 host threads (one per 128 Ki elements): the copies write
// disjoint destinations, so the threads share no output element.
template <class Put>
static void for_stack_elements(const std::vector<StackCopy>& jobs, Put put) {
    const int BK = kTcBK;
    struct Item { size_t job; int64_t r0, r1; };
    std::vector<Item> items;
    int64_t total = 0;
    const int64_t grain = 1 << 16;  // elements per work item
    for (size_t j = 0; j < jobs.size(); ++j) {
        const int64_t len = std::max<int64_t>(1, jobs[j].len);
        const int64_t step = std::max<int64_t>(1, grain / len);
        for (int64_t r0 = 0; r0 < jobs[j].nr; r0 += step) items.push_back({j, r0, std::min(jobs[j].nr, r0 + step)});
        total += jobs[j].nr * jobs[j].len;
    }
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (size_t it; (it = next.fetch_add(1)) < items.size();) {
            const StackCopy& c = jobs[items[it].job];
            for (int64_t r = items[it].r0; r < items[it].r1; ++r) {
                const double* src = c.src + r * c.len;
                for (int64_t kk = 0; kk < c.len; ++kk) {
                    const int64_t k = c.k_off + kk;
                    put((size_t)(c.row0 + (k / BK) * c.chunk_rows + r) * BK + (size_t)(k % BK), src[kk]);
                }
            }
        }
    };
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned nt = (unsigned)std::min<int64_t>(std::min(hw, 16u), std::max<int64_t>(1, total >> 17));
    std::vector<std::thread> pool;
    pool.reserve(nt);  // no reallocation (and no throw) once a thread runs
    for (unsigned t = 1; t < nt; ++t) {
        try {
            pool.emplace_back(work);
        } catch (const std::system_error&) {
            break;  // the calling thread still runs every remaining item
        }
    }
    work();
    for (std::thread& t : pool) t.join();
}

// Fills the bf16 hi / lo stacks of `rows` rows x kTcBK from the copy jobs:
// hi = bf16(v), lo = bf16(v - hi) (both rounded to nearest even through
// fp32), zero where no slab lands.  Jobs write disjoint elements, so row
// ranges of them run on several threads with the same result as one.
static void fill_split_stacks(const std::vector<StackCopy>& jobs, int64_t rows, std::vector<uint16_t>& hi,
                              std::vector<uint16_t>& lo) {
    hi.assign((size_t)rows * kTcBK, 0);
    lo.assign((size_t)rows * kTcBK, 0);
    uint16_t* H = hi.data();
    uint16_t* L = lo.data();
    for_stack_elements(jobs, [H, L](size_t at, double v) {
        const uint16_t h = f32_to_bf16_bits((float)v);
        H[at] = h;
        L[at] = f32_to_bf16_bits((float)(v - (double)bf16_bits_to_f32(h)));
    });
}

// The same stacks in FP64 (the stacked FP64 schedule): element for element
// the environment values, zero where no slab lands.
static void fill_stacks_f64(const std::vector<StackCopy>& jobs, int64_t rows, std::vector<double>& out) {
    out.assign((size_t)rows * kTcBK, 0.0);
    double* O = out.data();
    for_stack_elements(jobs, [O](size_t at, double v) { O[at] = v; });
}

// The split-precision (tensor-core) tables: both GEMM stages regrouped into
// operand stacks (see TcTables), built from the sector structure of the
// FP64 tables with the schedule options `o` (tall stage-1 stacks, fused stage
// 3).  Rebuilt alone when a plan changes its options.
static tk_status build_tc_tables(Heff2Tables& T, const TcSource& X, const TcOptions& o, TcTables& C, bool fp64,
                                 std::string& err, const double* lbuf_im = nullptr,
                                 const double* rbuf_im = nullptr) {
    using Term = TcSource::Term;
    const int nA = X.nA, nB = X.nB, nWL = X.nWL, nWR = X.nWR;
    const int64_t P = X.P, nwr = X.nwr;
    const QIndex &QA = X.QA, &QB = X.QB, &WL = X.WL, &WR = X.WR;
    const std::vector<int64_t>& lblk = X.lblk;
    const std::vector<int64_t>& rblk = X.rblk;
    const std::vector<std::vector<Term>>& byout = X.byout;
    const std::vector<int>& wl_sec = X.wl_sec;
    const std::vector<int64_t>& wl_loc = X.wl_loc;
    auto SUB = [&](int64_t p, int a, int b) -> int64_t { return X.sub[((size_t)p * nA + a) * nB + b]; };
    (void)WL;
    {
        C = TcTables();
        const int BK = kTcBK;
        auto kchunks = [&](int64_t K) { return (int32_t)((K + BK - 1) / BK); };
        std::vector<StackCopy> lcopy, rcopy;
        // T1 pieces: key (p, A', ws, B) -> (offset of channel-0 row, row stride per a')
        struct Piece { uint64_t key; int64_t off; int32_t rs; };
        std::vector<Piece> pieces;
        auto pkey = [&](int64_t p, int ap, int ws, int b) -> uint64_t {
            return (((uint64_t)p * nA + ap) * nWL + ws) * nB + b;
        };
        int64_t t1off = 0;
        std::vector<int64_t> tile1_xend;  // per tiles1 entry: end of the psi range it reads
        // stage 1: one stack per ket sector A
        for (int a = 0; a < nA; ++a) {
            std::vector<std::pair<int, int>> lp;   // (A', ws)
            std::vector<int64_t> lrow;
            int64_t rows = 0;
            for (int ap = 0; ap < nA; ++ap)
                for (int ws = 0; ws < nWL; ++ws)
                    if (lblk[((size_t)ap * nWL + ws) * nA + a] >= 0) {
                        lp.push_back({ap, ws});
                        lrow.push_back(rows);
                        rows += QA.dim[ap] * WL.dim[ws];
                    }
            std::vector<std::pair<int64_t, int>> xp;  // (p, B)
            for (int64_t p = 0; p < P; ++p)
                for (int b = 0; b < nB; ++b)
                    if (SUB(p, a, b) >= 0) xp.push_back({p, b});
            // columns in the order of their psi sub-blocks in the vector, so that
            // a tile's columns come from a narrow range of psi
            std::stable_sort(xp.begin(), xp.end(), [&](const std::pair<int64_t, int>& u, const std::pair<int64_t, int>& v) {
                return SUB(u.first, a, u.second) < SUB(v.first, a, v.second);
            });
            std::vector<int64_t> xcol;
            int64_t cols = 0;
            for (const auto& pb : xp) {
                xcol.push_back(cols);
                cols += QB.dim[pb.second];
            }
            if (rows == 0 || cols == 0) continue;
            const int64_t K = QA.dim[a];
            const int32_t kch = kchunks(K);
            const int64_t lb = C.lq_rows;
            C.lq_rows += kch * rows;
            for (size_t i = 0; i < lp.size(); ++i) {
                int ap = lp[i].first, ws = lp[i].second;
                lcopy.push_back({T.lbuf.data() + lblk[((size_t)ap * nWL + ws) * nA + a], QA.dim[ap] * WL.dim[ws], K, 0,
                                 lb + lrow[i], rows});
            }
            // T1 of this stack: one row-major [rows x D_B] matrix per column block (p, B);
            // the B operand column b of block (p, B) is column b of the psi sub-block (D_A x D_B)
            const int64_t colbase0 = (int64_t)C.t1col_base.size();
            for (size_t jx = 0; jx < xp.size(); ++jx) {
                const int64_t DB = QB.dim[xp[jx].second];
                const int64_t src = SUB(xp[jx].first, a, xp[jx].second);
                for (int64_t b = 0; b < DB; ++b) {
                    C.t1col_base.push_back(t1off + xcol[jx] * rows + b);
                    C.t1col_stride.push_back((int32_t)DB);
                    C.xsrc.push_back(src + b);
                    C.xstride.push_back((int32_t)DB);
                }
            }
            // tall stacks: psi split once into a bf16 copy (K-major chunks,
            // column b of block (p, B) on operand row xb + xcol + b of chunk 0)
            const bool tall = (rows + kTcBM - 1) / kTcBM > o.tall_max_mtiles;
            const int64_t xb = C.xq_rows;
            if (tall) {
                C.xq_rows += kch * cols;
                for (size_t jx = 0; jx < xp.size(); ++jx) {
                    TcSplitJob j{};
                    j.src = SUB(xp[jx].first, a, xp[jx].second);
                    j.rows = (int32_t)K;
                    j.cols = (int32_t)QB.dim[xp[jx].second];
                    j.xrow = (int32_t)(xb + xcol[jx]);
                    j.cstride = (int32_t)cols;
                    for (int32_t a0 = 0; a0 < j.rows; a0 += BK)
                        for (int32_t b0 = 0; b0 < j.cols; b0 += 32) {
                            j.a0 = a0;
                            j.b0 = b0;
                            C.split.push_back(j);
                        }
                }
            }
            for (int64_t m0 = 0; m0 < rows; m0 += kTcBM)
                for (int64_t n0 = 0; n0 < cols; n0 += kTcBN) {
                    TcTile t{};
                    t.a_row = (int32_t)(lb + m0); t.a_cs = (int32_t)rows;
                    t.b_row = tall ? (int32_t)(xb + n0) : 0;
                    t.b_cs = tall ? (int32_t)cols : 0;
                    t.k_valid = (int32_t)K;
                    t.kch = kch;
                    t.m_valid = (int32_t)std::min<int64_t>(kTcBM, rows - m0);
                    t.n_valid = (int32_t)std::min<int64_t>(kTcBN, cols - n0);
                    t.n_mma = (t.n_valid + 15) / 16 * 16;
                    t.mode = 2;
                    t.out_off = colbase0 + n0;
                    t.ldc = (int32_t)m0;
                    if (!tall) {
                        // end of the psi range the tile reads (its columns' sub-blocks)
                        int64_t xend = 0;
                        for (size_t jx = 0; jx < xp.size(); ++jx) {
                            const int64_t DB = QB.dim[xp[jx].second];
                            if (xcol[jx] < n0 + t.n_valid && xcol[jx] + DB > n0)
                                xend = std::max(xend, SUB(xp[jx].first, a, xp[jx].second) + K * DB);
                        }
                        tile1_xend.push_back(xend);
                    }
                    (tall ? C.tiles1x : C.tiles1).push_back(t);
                    C.mma_flops += 2.0 * kTcBM * t.n_mma * (double)kch * BK;
                }
            for (size_t i = 0; i < lp.size(); ++i)
                for (size_t jx = 0; jx < xp.size(); ++jx) {
                    const int64_t DB = QB.dim[xp[jx].second];
                    // channel-0 row of the slab, row stride per a' = dws rows of D_B
                    pieces.push_back({pkey(xp[jx].first, lp[i].first, lp[i].second, xp[jx].second),
                                      t1off + xcol[jx] * rows + lrow[i] * DB, (int32_t)(WL.dim[lp[i].second] * DB)});
                }
            t1off += rows * cols;
        }
        C.t1_total = t1off;
        std::sort(pieces.begin(), pieces.end(), [](const Piece& x, const Piece& y) { return x.key < y.key; });
        // stage 3: one stack per bra sector B' of R
        for (int bp = 0; bp < nB; ++bp) {
            std::vector<std::pair<int64_t, int>> yp;  // (p', A')
            std::vector<int64_t> yr;
            int64_t rows = 0;
            for (int64_t p = 0; p < P; ++p)
                for (int ap = 0; ap < nA; ++ap)
                    if (SUB(p, ap, bp) >= 0) {
                        yp.push_back({p, ap});
                        yr.push_back(rows);
                        rows += QA.dim[ap];
                    }
            if (rows == 0) continue;
            std::vector<std::pair<int, int>> rp;  // (ws, B)
            std::vector<int64_t> rk;
            int64_t K = 0;
            for (int ws = 0; ws < nWR; ++ws)
                for (int b = 0; b < nB; ++b)
                    if (rblk[((size_t)bp * nWR + ws) * nB + b] >= 0) {
                        rp.push_back({ws, b});
                        rk.push_back(K);
                        K += WR.dim[ws] * QB.dim[b];
                    }
            const int32_t kch = kchunks(K);
            const int64_t NB = QB.dim[bp];
            // the combine fused into the GEMM when the stack has few column tiles
            // (each column tile rebuilds the operand from T1)
            const bool fuse = (NB + kTcBN - 1) / kTcBN <= o.fuse_max_ntiles;
            const int64_t rbase = C.rq_rows, t2b = C.t2q_rows, yb = (int64_t)C.yrow.size();
            C.rq_rows += kch * NB;
            if (!fuse) C.t2q_rows += kch * rows;
            for (size_t i = 0; i < rp.size(); ++i) {
                int ws = rp[i].first, b = rp[i].second;
                rcopy.push_back({T.rbuf.data() + rblk[((size_t)bp * nWR + ws) * nB + b], NB, WR.dim[ws] * QB.dim[b], rk[i],
                                 rbase, NB});
            }
            // slabs of the A operand (T2): stack rows [row0, row0 + nr) x K columns
            // [k0, k0 + nc), element (r, c) = sum_t coef_t * T1[in_off_t + r * in_rs_t + c]
            struct Slab {
                int64_t row0;
                int32_t nr, k0, nc, tb, te;
            };
            std::vector<Slab> slabs;
            std::vector<TcCombTerm> sterms;
            std::vector<double> scoef;  // the same coefficients in FP64
            for (size_t i = 0; i < yp.size(); ++i) {
                int64_t po = yp[i].first;
                int ap = yp[i].second;
                int64_t yo = SUB(po, ap, bp);
                for (int64_t r = 0; r < QA.dim[ap]; ++r) C.yrow.push_back(yo + r * NB);
                for (size_t ri = 0; ri < rp.size(); ++ri) {
                    int ws = rp[ri].first, b = rp[ri].second;
                    for (int64_t wloc = 0; wloc < WR.dim[ws]; ++wloc) {
                        int64_t wr = WR.off[ws] + wloc;
                        Slab sl{yr[i], (int32_t)QA.dim[ap], (int32_t)(rk[ri] + wloc * QB.dim[b]), (int32_t)QB.dim[b],
                                (int32_t)sterms.size(), 0};
                        for (const Term& tm : byout[po * nwr + wr]) {
                            uint64_t key = pkey(tm.p, ap, wl_sec[tm.wl], b);
                            auto it = std::lower_bound(pieces.begin(), pieces.end(), key,
                                                       [](const Piece& x, uint64_t k) { return x.key < k; });
                            for (; it != pieces.end() && it->key == key; ++it) {
                                TcCombTerm ct{};
                                ct.in_off = it->off + wl_loc[tm.wl] * (int64_t)(it->rs / WL.dim[wl_sec[tm.wl]]);
                                ct.in_rs = it->rs;
                                ct.coef = (float)tm.c;
                                sterms.push_back(ct);
                                scoef.push_back(tm.c);
                            }
                        }
                        sl.te = (int32_t)sterms.size();
                        if (sl.te > sl.tb) slabs.push_back(sl);
                    }
                }
            }
            if (!fuse) {
                // combine jobs: rows of one slab, at most kTcCombMaxElems elements each
                for (const Slab& sl : slabs) {
                    TcCombJob j{};
                    j.t2row = (int32_t)(t2b + sl.row0);
                    j.cstride = (int32_t)rows;
                    j.k0 = sl.k0;
                    j.cols = sl.nc;
                    j.term_begin = (int32_t)C.terms.size();
                    C.terms.insert(C.terms.end(), sterms.begin() + sl.tb, sterms.begin() + sl.te);
                    C.term_coef64.insert(C.term_coef64.end(), scoef.begin() + sl.tb, scoef.begin() + sl.te);
                    j.term_end = (int32_t)C.terms.size();
                    for (int q = 0; q < kTcCombInline && j.term_begin + q < j.term_end; ++q)
                        j.inl[q] = C.terms[j.term_begin + q];
                    const int32_t step = std::max<int32_t>(1, kTcCombMaxElems / std::max<int32_t>(1, j.cols));
                    for (int32_t r0 = 0; r0 < sl.nr; r0 += step) {
                        j.r0 = r0;
                        j.rows = std::min(step, sl.nr - r0);
                        C.jobs.push_back(j);
                    }
                }
            }
            for (int64_t m0 = 0; m0 < rows; m0 += kTcBM) {
                int32_t fill0 = -1;
                if (fuse) {
                    // fill segments of this row tile, chunk by chunk: every slab part
                    // inside rows [m0, m0 + 128) and K chunk [64c, 64c + 64)
                    fill0 = (int32_t)C.fill_chunk.size();
                    for (int32_t c = 0; c < kch; ++c) {
                        C.fill_chunk.push_back((int32_t)C.fill_segs.size());
                        const int64_t ka = (int64_t)c * BK, kb = ka + BK;
                        for (const Slab& sl : slabs) {
                            const int64_t ra = std::max<int64_t>(sl.row0, m0);
                            const int64_t rb = std::min<int64_t>(sl.row0 + sl.nr, m0 + kTcBM);
                            const int64_t c0 = std::max<int64_t>(sl.k0, ka), c1 = std::min<int64_t>(sl.k0 + sl.nc, kb);
                            if (ra >= rb || c0 >= c1) continue;
                            TcFillSeg g{};
                            g.r0 = (int16_t)(ra - m0);
                            g.rows = (int16_t)(rb - ra);
                            g.k0 = (int16_t)(c0 - ka);
                            g.cols = (int16_t)(c1 - c0);
                            g.term_begin = (int32_t)C.fill_terms.size();
                            for (int32_t t = sl.tb; t < sl.te; ++t) {
                                TcCombTerm ct = sterms[t];
                                ct.in_off += (ra - sl.row0) * (int64_t)ct.in_rs + (c0 - sl.k0);
                                C.fill_terms.push_back(ct);
                            }
                            g.term_end = (int32_t)C.fill_terms.size();
                            C.fill_term_elems += (double)g.rows * g.cols * (g.term_end - g.term_begin);
                            C.fill_segs.push_back(g);
                        }
                    }
                    C.fill_chunk.push_back((int32_t)C.fill_segs.size());
                }
                for (int64_t n0 = 0; n0 < NB; n0 += kTcBN) {
                    TcTile t{};
                    t.a_row = fuse ? 0 : (int32_t)(t2b + m0);
                    t.a_cs = fuse ? 0 : (int32_t)rows;
                    t.b_row = (int32_t)(rbase + n0); t.b_cs = (int32_t)NB;
                    t.kch = kch;
                    t.k_valid = (int32_t)K;
                    t.m_valid = (int32_t)std::min<int64_t>(kTcBM, rows - m0);
                    t.n_valid = (int32_t)std::min<int64_t>(kTcBN, NB - n0);
                    t.n_mma = (t.n_valid + 15) / 16 * 16;
                    t.mode = fuse ? 3 : 1;
                    t.out_off = yb + m0;
                    t.ldc = 0;
                    t.n0 = (int32_t)n0;
                    t.fill0 = fill0;
                    (fuse ? C.tiles3f : C.tiles3).push_back(t);
                    C.mma_flops += 2.0 * kTcBM * t.n_mma * (double)kch * BK;
                }
            }
        }
        // heaviest tiles first (K chunks, then padded MMA area): a launch with
        // more tiles than resident CTAs ends on a tail of light tiles
        // (LPT order, as tk-linalg/src/tasks.rs:172-174 orders sector tasks)
        auto lpt = [](std::vector<TcTile>& v) {
            std::stable_sort(v.begin(), v.end(), [](const TcTile& a, const TcTile& b) {
                if (a.kch != b.kch) return a.kch > b.kch;
                return (int64_t)a.m_valid * a.n_mma > (int64_t)b.m_valid * b.n_mma;
            });
        };
        // psi in kTcPsiPieces pieces (block boundaries near equal shares): the
        // in-GEMM-split tiles go in the order of the piece their last psi read
        // falls in, so a host-buffer matvec can start each group as soon as its
        // piece is on the device while the later pieces are still being copied
        {
            constexpr int KP = kTcPsiPieces;
            C.x_cut[0] = 0;
            C.x_cut[KP] = T.total;
            size_t bi = 0;
            for (int j = 1; j < KP; ++j) {
                while (bi < T.blk_off.size() && (int64_t)KP * T.blk_off[bi] < (int64_t)j * T.total) ++bi;
                C.x_cut[j] = bi < T.blk_off.size() ? T.blk_off[bi] : T.total;
            }
            std::vector<std::vector<TcTile>> groups(KP);
            for (size_t i = 0; i < C.tiles1.size(); ++i) {
                int j = 0;
                while (j < KP - 1 && tile1_xend[i] > C.x_cut[j + 1]) ++j;
                groups[(size_t)j].push_back(C.tiles1[i]);
            }
            C.tiles1.clear();
            C.n1_cut[0] = 0;
            for (int j = 0; j < KP; ++j) {
                lpt(groups[(size_t)j]);
                C.tiles1.insert(C.tiles1.end(), groups[(size_t)j].begin(), groups[(size_t)j].end());
                C.n1_cut[j + 1] = (int32_t)C.tiles1.size();
            }
        }
        lpt(C.tiles1x);
        lpt(C.tiles3);
        lpt(C.tiles3f);
        for (const TcTile& t : C.tiles1) C.max_kch1 = std::max(C.max_kch1, t.kch);
        for (const TcTile& t : C.tiles1x) C.max_kch1x = std::max(C.max_kch1x, t.kch);
        for (const TcTile& t : C.tiles3) C.max_kch3 = std::max(C.max_kch3, t.kch);
        for (const TcTile& t : C.tiles3f) C.max_kch3f = std::max(C.max_kch3f, t.kch);
        // the constant operands as bf16 hi + lo stacks
        host_alloc_checkpoint();
        if (fp64) {
            fill_stacks_f64(lcopy, C.lq_rows, C.lq64);
            fill_stacks_f64(rcopy, C.rq_rows, C.rq64);
            if (lbuf_im && rbuf_im) {
                // imaginary parts of complex environments: the same copies from the
                // same offsets of the imaginary slab arrays
                std::vector<StackCopy> li(lcopy), ri(rcopy);
                for (StackCopy& c : li) c.src = lbuf_im + (c.src - T.lbuf.data());
                for (StackCopy& c : ri) c.src = rbuf_im + (c.src - T.rbuf.data());
                fill_stacks_f64(li, C.lq_rows, C.lq64_im);
                fill_stacks_f64(ri, C.rq_rows, C.rq64_im);
            }
        } else {
            fill_split_stacks(lcopy, C.lq_rows, C.lq_hi, C.lq_lo);
            fill_split_stacks(rcopy, C.rq_rows, C.rq_hi, C.rq_lo);
        }
        if (C.lq_rows > INT32_MAX || C.rq_rows > INT32_MAX || C.xq_rows > INT32_MAX || C.t2q_rows > INT32_MAX) {
            err = "tensor-core operand rows exceed 32 bits";
            return TK_ERR_UNSUPPORTED;
        }
        }
    return TK_OK;
}

static tk_status build_heff2_tables_body(const tk_env& envL, const tk_env& envR, const tk_bst& wi_abi,
                                         const tk_bst& wj_abi, const int32_t* psi_flux, int tile_m, int tile_n,
                                         Heff2Tables& T, std::string& err, const double* l_blocks,
                                         const double* r_blocks) {
    Bst4 wi, wj;
    if (!bst4_from_abi(wi_abi, wi, "W_i", err)) return TK_ERR_INVALID_ARG;
    if (!bst4_from_abi(wj_abi, wj, "W_j", err)) return TK_ERR_INVALID_ARG;
    if (wi.kind != wj.kind) {
        err = "W_i and W_j use different quantum-number kinds";
        return TK_ERR_INVALID_ARG;
    }
    const int kind = wi.kind;
    T.kind = kind;
    QIndex lbra, lmpo, lket, rbra, rmpo, rket;
    if (!qindex_from_abi(kind, envL.bra, lbra, err) || !qindex_from_abi(kind, envL.mpo, lmpo, err) ||
        !qindex_from_abi(kind, envL.ket, lket, err) || !qindex_from_abi(kind, envR.bra, rbra, err) ||
        !qindex_from_abi(kind, envR.mpo, rmpo, err) || !qindex_from_abi(kind, envR.ket, rket, err)) {
        err = "environment: " + err;
        return TK_ERR_INVALID_ARG;
    }
    if (!envL.data || !envR.data) {
        err = "environment: null data";
        return TK_ERR_INVALID_ARG;
    }
    // The reference loops a'_L over the ket dimension (mod.rs:503, :559): the
    // bra and ket bases must agree.
    if (!lbra.same_as(lket) || !rbra.same_as(rket)) {
        err = "environment bra and ket QIndex differ";
        return TK_ERR_SECTOR_MISMATCH;
    }
    if (!wi.legs[0].same_as(wi.legs[1]) || !wj.legs[0].same_as(wj.legs[1])) {
        err = "MPO s_in and s_out QIndex differ";
        return TK_ERR_SECTOR_MISMATCH;
    }
    if (!wi.legs[2].same_as(lmpo) || !wj.legs[3].same_as(rmpo)) {
        err = "MPO bond QIndex does not match the environment's MPO leg";
        return TK_ERR_SECTOR_MISMATCH;
    }
    if (!wi.legs[3].same_as(wj.legs[2])) {
        err = "W_i right bond and W_j left bond QIndex differ";
        return TK_ERR_SECTOR_MISMATCH;
    }
    const QIndex& PI = wi.legs[0];
    const QIndex& PJ = wj.legs[0];
    const QIndex& QA = lket;
    const QIndex& QB = rket;
    const QIndex& WL = lmpo;
    const QIndex& WR = rmpo;
    const int64_t d_i = PI.total, d_j = PJ.total, d_l = QA.total, d_r = QB.total;
    const int64_t nwl = WL.total, nwm = wi.legs[3].total, nwr = WR.total;
    T.d_i = d_i; T.d_j = d_j; T.d_l = d_l; T.d_r = d_r; T.nwl = nwl; T.nwr = nwr;
    const int nA = QA.n(), nB = QB.n();
    const int64_t P = d_i * d_j;

    // --- fused two-site operator W_ij[p][p'][wl][wr] = sum_wm W_i W_j ---------
    std::vector<double> Wi, Wj;
    if (!mpo_dense(wi, Wi, err) || !mpo_dense(wj, Wj, err)) return TK_ERR_SECTOR_MISMATCH;
    host_alloc_checkpoint();
    std::vector<double> Wij((size_t)(P * P * nwl * nwr), 0.0);
    for (int64_t si = 0; si < d_i; ++si)
        for (int64_t so = 0; so < d_i; ++so)
            for (int64_t sj = 0; sj < d_j; ++sj)
                for (int64_t to = 0; to < d_j; ++to)
                    for (int64_t wl = 0; wl < nwl; ++wl)
                        for (int64_t wm = 0; wm < nwm; ++wm) {
                            double a = Wi[((si * d_i + so) * nwl + wl) * nwm + wm];
                            if (a == 0.0) continue;
                            for (int64_t wr = 0; wr < nwr; ++wr) {
                                double b = Wj[((sj * d_j + to) * nwm + wm) * nwr + wr];
                                if (b == 0.0) continue;
                                Wij[(((si * d_j + sj) * P + (so * d_j + to)) * nwl + wl) * nwr + wr] += a * b;
                            }
                        }

    // --- two-site blocks ---------------------------------------------------------
    std::vector<std::array<int, 4>> tuples;
    QIndex legs4[4] = {PI, PJ, QA, QB};
    if (psi_flux) {
        Qn f;
        for (int k = 0; k < qn_ncomp(kind); ++k) f.c[k] = psi_flux[k];
        enumerate4(kind, legs4, f, tuples);
    } else {
        for (int a = 0; a < PI.n(); ++a)
            for (int b = 0; b < PJ.n(); ++b)
                for (int c = 0; c < nA; ++c)
                    for (int d = 0; d < nB; ++d) tuples.push_back({a, b, c, d});
    }
    if (4 * qn_bits(kind) > 64) {
        err = "rank-4 sector key exceeds 64 bits";
        return TK_ERR_UNSUPPORTED;
    }
    std::vector<std::pair<uint64_t, std::array<int, 4>>> kb;
    kb.reserve(tuples.size());
    for (auto& t : tuples) {
        Qn q[4] = {PI.q[t[0]], PJ.q[t[1]], QA.q[t[2]], QB.q[t[3]]};
        kb.push_back({key_pack(kind, q, 4), t});
    }
    std::sort(kb.begin(), kb.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    // state -> (sector, local)
    std::vector<int> secI(d_i), secJ(d_j);
    std::vector<int64_t> locI(d_i), locJ(d_j);
    for (int s = 0; s < PI.n(); ++s)
        for (int64_t k = 0; k < PI.dim[s]; ++k) { secI[PI.off[s] + k] = s; locI[PI.off[s] + k] = k; }
    for (int s = 0; s < PJ.n(); ++s)
        for (int64_t k = 0; k < PJ.dim[s]; ++k) { secJ[PJ.off[s] + k] = s; locJ[PJ.off[s] + k] = k; }

    // sub-block (p, A, B) -> flat offset
    std::vector<int64_t> sub((size_t)(P * nA * nB), -1);
    auto SUB = [&](int64_t p, int a, int b) -> int64_t& { return sub[((size_t)p * nA + a) * nB + b]; };
    T.keys.clear();
    T.blk_off.clear();
    T.submaps.clear();
    int64_t off = 0;
    for (auto& e : kb) {
        const auto& t = e.second;
        T.keys.push_back(e.first);
        T.blk_off.push_back(off);
        int64_t ni = PI.dim[t[0]], nj = PJ.dim[t[1]], DA = QA.dim[t[2]], DB = QB.dim[t[3]];
        for (int64_t li = 0; li < ni; ++li)
            for (int64_t lj = 0; lj < nj; ++lj) {
                int64_t p = (PI.off[t[0]] + li) * d_j + (PJ.off[t[1]] + lj);
                int64_t fo = off + (li * nj + lj) * DA * DB;
                SUB(p, t[2], t[3]) = fo;
                T.submaps.push_back({p * d_l * d_r + QA.off[t[2]] * d_r + QB.off[t[3]], fo, (int32_t)DA, (int32_t)DB});
            }
        off += ni * nj * DA * DB;
    }
    T.total = off;

    host_alloc_checkpoint();
    // --- non-zero environment slabs -------------------------------------------
    // L slab (A', ws, A) as [(a', w)][a]; R slab (B', ws, B) as [b'][(w, b)].
    const int nWL = WL.n(), nWR = WR.n();
    std::vector<int64_t> lblk((size_t)nA * nWL * nA, -1), rblk((size_t)nB * nWR * nB, -1);
    T.lbuf.clear();
    T.rbuf.clear();
    if (l_blocks) {
        // canonical block layout: every charge-allowed block is a slab, in place
        EnvLayout lay;
        env_layout(kind, QA, WL, QA, lay);
        for (size_t k = 0; k < lay.tri.size(); ++k)
            lblk[((size_t)lay.tri[k][0] * nWL + lay.tri[k][1]) * nA + lay.tri[k][2]] = lay.off[k];
        T.lbuf.assign(l_blocks, l_blocks + lay.total);
    }
    if (r_blocks) {
        EnvLayout lay;
        env_layout(kind, QB, WR, QB, lay);
        for (size_t k = 0; k < lay.tri.size(); ++k)
            rblk[((size_t)lay.tri[k][0] * nWR + lay.tri[k][1]) * nB + lay.tri[k][2]] = lay.off[k];
        T.rbuf.assign(r_blocks, r_blocks + lay.total);
    }
    for (int ap = 0; ap < nA && !l_blocks; ++ap)
        for (int ws = 0; ws < nWL; ++ws)
            for (int a = 0; a < nA; ++a) {
                bool nz = false;
                for (int64_t i = 0; i < QA.dim[ap] && !nz; ++i)
                    for (int64_t w = 0; w < WL.dim[ws] && !nz; ++w) {
                        const double* row = envL.data + ((QA.off[ap] + i) * nwl + WL.off[ws] + w) * d_l + QA.off[a];
                        for (int64_t j = 0; j < QA.dim[a]; ++j)
                            if (row[j] != 0.0) { nz = true; break; }
                    }
                if (!nz) continue;
                lblk[((size_t)ap * nWL + ws) * nA + a] = (int64_t)T.lbuf.size();
                for (int64_t i = 0; i < QA.dim[ap]; ++i)
                    for (int64_t w = 0; w < WL.dim[ws]; ++w) {
                        const double* row = envL.data + ((QA.off[ap] + i) * nwl + WL.off[ws] + w) * d_l + QA.off[a];
                        T.lbuf.insert(T.lbuf.end(), row, row + QA.dim[a]);
                    }
            }
    for (int bp = 0; bp < nB && !r_blocks; ++bp)
        for (int ws = 0; ws < nWR; ++ws)
            for (int b = 0; b < nB; ++b) {
                bool nz = false;
                for (int64_t i = 0; i < QB.dim[bp] && !nz; ++i)
                    for (int64_t w = 0; w < WR.dim[ws] && !nz; ++w) {
                        const double* row = envR.data + ((QB.off[bp] + i) * nwr + WR.off[ws] + w) * d_r + QB.off[b];
                        for (int64_t j = 0; j < QB.dim[b]; ++j)
                            if (row[j] != 0.0) { nz = true; break; }
                    }
                if (!nz) continue;
                rblk[((size_t)bp * nWR + ws) * nB + b] = (int64_t)T.rbuf.size();
                for (int64_t i = 0; i < QB.dim[bp]; ++i)
                    for (int64_t w = 0; w < WR.dim[ws]; ++w) {
                        const double* row = envR.data + ((QB.off[bp] + i) * nwr + WR.off[ws] + w) * d_r + QB.off[b];
                        T.rbuf.insert(T.rbuf.end(), row, row + QB.dim[b]);
                    }
            }

    host_alloc_checkpoint();
    // --- stage 1: T1(p, A', ws, B) = sum_A Lslab(A', ws, A) * psi(p, A, B) -----
    std::vector<int64_t> t1((size_t)P * nA * nWL * nB, -1);
    auto T1I = [&](int64_t p, int ap, int ws, int b) -> int64_t& {
        return t1[(((size_t)p * nA + ap) * nWL + ws) * nB + b];
    };
    // ket sectors A of the L slabs (A', ws, A), ascending; charge conservation
    // leaves at most a few per (A', ws), so the task scan below stays linear
    std::vector<std::vector<int>> lslab_ket((size_t)nA * nWL);
    for (int ap = 0; ap < nA; ++ap)
        for (int ws = 0; ws < nWL; ++ws)
            for (int a = 0; a < nA; ++a)
                if (lblk[((size_t)ap * nWL + ws) * nA + a] >= 0) lslab_ket[(size_t)ap * nWL + ws].push_back(a);
    T.g1 = GemmTable();
    off = 0;
    for (int64_t p = 0; p < P; ++p)
        for (int ap = 0; ap < nA; ++ap)
            for (int ws = 0; ws < nWL; ++ws)
                for (int b = 0; b < nB; ++b) {
                    int seg0 = (int)T.g1.segs.size();
                    std::vector<int64_t> ks;
                    for (int a : lslab_ket[(size_t)ap * nWL + ws]) {
                        int64_t lo = lblk[((size_t)ap * nWL + ws) * nA + a];
                        int64_t so = SUB(p, a, b);
                        if (so < 0) continue;
                        GemmSeg s{};
                        s.a_off = lo; s.a_rs = (int32_t)QA.dim[a]; s.a_cs = 1;
                        s.b_off = so; s.b_rs = (int32_t)QB.dim[b]; s.b_cs = 1;
                        s.K = (int32_t)QA.dim[a];
                        T.g1.segs.push_back(s);
                        ks.push_back(s.K);
                    }
                    if (ks.empty()) continue;
                    GemmTask tk{};
                    tk.M = (int32_t)(QA.dim[ap] * WL.dim[ws]);
                    tk.N = (int32_t)QB.dim[b];
                    tk.c_off = off; tk.c_rs = tk.N; tk.c_cs = 1;
                    tk.seg_begin = seg0; tk.seg_end = (int)T.g1.segs.size();
                    tk.alpha = 1.0; tk.beta = 0.0;
                    for (int64_t k : ks) T.g1.flops += 2.0 * tk.M * tk.N * (double)k;
                    T1I(p, ap, ws, b) = off;
                    off += (int64_t)tk.M * tk.N;
                    T.g1.tasks.push_back(tk);
                    add_tiles(T.g1, (int)T.g1.tasks.size() - 1, tile_m, tile_n, ks);
                }
    T.t1_total = off;

    host_alloc_checkpoint();
    // --- stage 2: T2(p', A', wsr, B)[a'][w][b] = sum W_ij * T1 -----------------
    std::vector<int> wl_sec(nwl), wr_sec(nwr);
    std::vector<int64_t> wl_loc(nwl), wr_loc(nwr);
    for (int s = 0; s < nWL; ++s)
        for (int64_t k = 0; k < WL.dim[s]; ++k) { wl_sec[WL.off[s] + k] = s; wl_loc[WL.off[s] + k] = k; }
    for (int s = 0; s < nWR; ++s)
        for (int64_t k = 0; k < WR.dim[s]; ++k) { wr_sec[WR.off[s] + k] = s; wr_loc[WR.off[s] + k] = k; }
    // non-zero W_ij terms grouped by (p', wr)
    using Term = TcSource::Term;
    std::vector<std::vector<Term>> byout((size_t)(P * nwr));
    int64_t nterms = 0;
    for (int64_t p = 0; p < P; ++p)
        for (int64_t po = 0; po < P; ++po)
            for (int64_t wl = 0; wl < nwl; ++wl)
                for (int64_t wr = 0; wr < nwr; ++wr) {
                    double c = Wij[((p * P + po) * nwl + wl) * nwr + wr];
                    if (c != 0.0) { byout[po * nwr + wr].push_back({p, wl, c}); ++nterms; }
                }
    T.n_wij_terms = nterms;
    std::vector<int64_t> t2((size_t)P * nA * nWR * nB, -1);
    auto T2I = [&](int64_t p, int ap, int ws, int b) -> int64_t& {
        return t2[(((size_t)p * nA + ap) * nWR + ws) * nB + b];
    };
    // bra sectors B' of the R slabs (B', ws, B), ascending
    std::vector<std::vector<int>> rslab_bra((size_t)nWR * nB);
    for (int bp = 0; bp < nB; ++bp)
        for (int ws = 0; ws < nWR; ++ws)
            for (int b = 0; b < nB; ++b)
                if (rblk[((size_t)bp * nWR + ws) * nB + b] >= 0) rslab_bra[(size_t)ws * nB + b].push_back(bp);
    T.jobs.clear();
    T.terms.clear();
    T.comb_flops = 0.0;
    off = 0;
    for (int64_t po = 0; po < P; ++po)
        for (int ap = 0; ap < nA; ++ap)
            for (int ws = 0; ws < nWR; ++ws)
                for (int b = 0; b < nB; ++b) {
                    // consumed by stage 3 only if some R slab (B', ws, B) exists and
                    // the output sub-block (p', A', B') exists
                    bool used = false;
                    for (int bp : rslab_bra[(size_t)ws * nB + b])
                        if (SUB(po, ap, bp) >= 0) {
                            used = true;
                            break;
                        }
                    if (!used) continue;
                    int64_t dws = WR.dim[ws];
                    size_t job0 = T.jobs.size();
                    bool any = false;
                    for (int64_t wlc = 0; wlc < dws; ++wlc) {
                        int64_t wr = WR.off[ws] + wlc;
                        CombJob j{};
                        j.rows = (int32_t)QA.dim[ap];
                        j.cols = (int32_t)QB.dim[b];
                        j.term_begin = (int32_t)T.terms.size();
                        for (const Term& tm : byout[po * nwr + wr]) {
                            int64_t src = T1I(tm.p, ap, wl_sec[tm.wl], b);
                            if (src < 0) continue;
                            CombTerm ct{};
                            ct.in_off = src + wl_loc[tm.wl] * QB.dim[b];
                            ct.in_rs = (int32_t)(WL.dim[wl_sec[tm.wl]] * QB.dim[b]);
                            ct.coef = tm.c;
                            T.terms.push_back(ct);
                            T.comb_flops += 2.0 * j.rows * j.cols;
                        }
                        j.term_end = (int32_t)T.terms.size();
                        if (j.term_end > j.term_begin) any = true;
                        j.out_off = wlc * QB.dim[b];  // relative; fixed below
                        j.out_rs = (int32_t)(dws * QB.dim[b]);
                        T.jobs.push_back(j);
                    }
                    if (!any) {
                        T.terms.resize(T.jobs[job0].term_begin);
                        T.jobs.resize(job0);
                        continue;
                    }
                    for (size_t k = job0; k < T.jobs.size(); ++k) T.jobs[k].out_off += off;
                    T2I(po, ap, ws, b) = off;
                    off += QA.dim[ap] * dws * QB.dim[b];
                }
    T.t2_total = off;

    host_alloc_checkpoint();
    // --- stage 3: y(p', A', B') = sum_{ws, B} T2(p', A', ws, B) * Rslab(B', ws, B)^T
    T.g3 = GemmTable();
    for (int64_t po = 0; po < P; ++po)
        for (int ap = 0; ap < nA; ++ap)
            for (int bp = 0; bp < nB; ++bp) {
                int64_t yo = SUB(po, ap, bp);
                if (yo < 0) continue;
                int seg0 = (int)T.g3.segs.size();
                std::vector<int64_t> ks;
                for (int ws = 0; ws < nWR; ++ws)
                    for (int b = 0; b < nB; ++b) {
                        int64_t ro = rblk[((size_t)bp * nWR + ws) * nB + b];
                        int64_t to = T2I(po, ap, ws, b);
                        if (ro < 0 || to < 0) continue;
                        int32_t K = (int32_t)(WR.dim[ws] * QB.dim[b]);
                        GemmSeg s{};
                        s.a_off = to; s.a_rs = K; s.a_cs = 1;
                        s.b_off = ro; s.b_rs = 1; s.b_cs = K;
                        s.K = K;
                        T.g3.segs.push_back(s);
                        ks.push_back(K);
                    }
                GemmTask tk{};
                tk.M = (int32_t)QA.dim[ap];
                tk.N = (int32_t)QB.dim[bp];
                tk.c_off = yo; tk.c_rs = tk.N; tk.c_cs = 1;
                tk.seg_begin = seg0; tk.seg_end = (int)T.g3.segs.size();
                tk.alpha = 1.0; tk.beta = 0.0;
                for (int64_t k : ks) T.g3.flops += 2.0 * tk.M * tk.N * (double)k;
                T.g3.tasks.push_back(tk);
                add_tiles(T.g3, (int)T.g3.tasks.size() - 1, tile_m, tile_n, ks);
            }
    // --- split-precision regrouping (tensor-core stacks) ---------------------
    {
        auto X = std::make_shared<TcSource>();
        X->nA = nA; X->nB = nB; X->nWL = nWL; X->nWR = nWR; X->P = P; X->nwr = nwr;
        X->QA = QA; X->QB = QB; X->WL = WL; X->WR = WR;
        X->lblk = std::move(lblk);
        X->rblk = std::move(rblk);
        X->sub = std::move(sub);
        X->byout = std::move(byout);
        X->wl_sec = wl_sec;
        X->wl_loc = wl_loc;
        T.tcsrc = X;  // the split tables themselves are built on first use (ensure_tc_tables)
    }
    lpt_order(T.g1, tile_m, tile_n);
    lpt_order(T.g3, tile_m, tile_n);
    // Algorithmic bytes: psi in, y out, the block-sparse L, R and W_ij terms, FP64.
    T.alg_bytes = 8.0 * (2.0 * (double)T.total + (double)T.lbuf.size() + (double)T.rbuf.size() + (double)nterms);
    // Index ranges must fit the kernels' 32-bit strides and counts.
    if (T.g1.tiles.size() > (size_t)INT32_MAX || T.g3.tiles.size() > (size_t)INT32_MAX ||
        T.terms.size() > (size_t)INT32_MAX || T.g1.segs.size() > (size_t)INT32_MAX) {
        err = "sector tables exceed 32-bit index range";
        return TK_ERR_UNSUPPORTED;
    }
    if (!validate_tables(T, err)) {
        err = "internal table check failed: " + err;
        return TK_ERR_INVALID_ARG;
    }
    return TK_OK;
}

}  // namespace tk

namespace tk {

tk_status build_f64_stacks(Heff2Tables& T, std::string& err, const double* lbuf_im, const double* rbuf_im) {
    if (!T.tcsrc) {
        err = "the plan keeps no sector structure to build from";
        return TK_ERR_UNSUPPORTED;
    }
    return guard_host("stacked FP64 tables", err, [&]() -> tk_status {
        TcOptions o;
        o.tall_max_mtiles = 1 << 30;  // every stage-1 column read from psi through its table
        o.fuse_max_ntiles = 0;        // every stage-3 stack reads a combined T2
        TcTables C;
        tk_status st = build_tc_tables(T, *T.tcsrc, o, C, true, err, lbuf_im, rbuf_im);
        if (st == TK_OK && !validate_tc(T, C, err)) {
            err = "internal table check failed: " + err;
            st = TK_ERR_INVALID_ARG;
        }
        if (st == TK_OK) T.f64st = std::move(C);
        return st;
    });
}

tk_status ensure_tc_tables(Heff2Tables& T, std::string& err) {
    if (T.tc_built) return TK_OK;
    if (!T.tcsrc) {
        err = "the plan keeps no sector structure to build from";
        return TK_ERR_UNSUPPORTED;
    }
    return guard_host("split-precision tables", err, [&]() -> tk_status {
        tk_status st = build_tc_tables(T, *T.tcsrc, T.tcopt, T.tc, false, err);
        if (st == TK_OK && !validate_tc(T, T.tc, err)) {
            err = "internal table check failed: " + err;
            st = TK_ERR_INVALID_ARG;
        }
        if (st == TK_OK)
            T.tc_built = true;
        else
            T.tc = TcTables();
        return st;
    });
}

tk_status rebuild_tc_tables(Heff2Tables& T, const TcOptions& o, std::string& err) {
    if (!T.tcsrc) {
        err = "the plan keeps no sector structure to rebuild from";
        return TK_ERR_UNSUPPORTED;
    }
    return guard_host("split-precision tables", err, [&]() -> tk_status {
        TcTables saved = std::move(T.tc);
        const TcOptions old = T.tcopt;
        const bool was_built = T.tc_built;
        T.tcopt = o;
        T.tc_built = true;
        tk_status st = build_tc_tables(T, *T.tcsrc, o, T.tc, false, err);
        if (st == TK_OK && !validate_tables(T, err)) {
            err = "internal table check failed: " + err;
            st = TK_ERR_INVALID_ARG;
        }
        if (st != TK_OK) {
            T.tc = std::move(saved);
            T.tcopt = old;
            T.tc_built = was_built;
        }
        return st;
    });
}

}  // namespace tk

extern "C" void tk_debug_fail_host_alloc(int32_t countdown) {
    tk::g_fail_host_alloc.store(countdown > 0 ? countdown : 0, std::memory_order_relaxed);
}

namespace tk {

tk_status build_heff2_tables(const tk_env& envL, const tk_env& envR, const tk_bst& wi_abi, const tk_bst& wj_abi,
                             const int32_t* psi_flux, int tile_m, int tile_n, Heff2Tables& T, std::string& err,
                             const double* l_blocks, const double* r_blocks) {
    return guard_host("sector tables", err, [&] {
        return build_heff2_tables_body(envL, envR, wi_abi, wj_abi, psi_flux, tile_m, tile_n, T, err, l_blocks, r_blocks);
    });
}

}  // namespace tk
