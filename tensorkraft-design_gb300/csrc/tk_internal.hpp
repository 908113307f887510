// tk_internal.hpp -- shared types of libtk_heff: quantum-number arithmetic,
// flattened sector-GEMM task tables, and the host-side plan description.
#pragma once
#include <algorithm>
#include <array>
#include <cstdint>
#include <cstring>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/tk_heff.h"

// Library context: the CUDA device it is bound to, the cuSOLVER handle of
// the dense factorisations (created on first use), and the grow-only scratch
// of the backend calls (block_gemm, spmv, gemm, pairwise contraction): one
// device arena, one page-locked host staging buffer and a stream, so that
// repeated calls allocate nothing once the arena has reached their size.
struct tk_ctx {
    int device = 0;
    void* solver = nullptr;
    void* dev_scratch = nullptr;
    size_t dev_scratch_bytes = 0;
    void* host_stage = nullptr;
    size_t host_stage_bytes = 0;
    void* stream = nullptr;  // cudaStream_t
};

namespace tk {

// ---------------------------------------------------------------------------
// Quantum numbers.  Semantics of tk-symmetry/src/builtins.rs:12-152: U(1)
// components add and negate, Z2 components xor and are self-dual; packing
// truncates each U(1) component to its bit field (Rust `as u8` / `as u16`).
// Order is lexicographic over components (derived Ord on the tuple structs).
// ---------------------------------------------------------------------------
struct Qn {
    int32_t c[2] = {0, 0};
    bool operator==(const Qn& o) const { return c[0] == o.c[0] && c[1] == o.c[1]; }
    bool operator!=(const Qn& o) const { return !(*this == o); }
};

int qn_ncomp(int kind);
int qn_bits(int kind);
bool qn_kind_valid(int kind);
Qn qn_fuse(int kind, const Qn& a, const Qn& b);
Qn qn_dual(int kind, const Qn& a);
bool qn_less(const Qn& a, const Qn& b);
uint64_t qn_pack(int kind, const Qn& q);
Qn qn_unpack(int kind, uint64_t bits);
// PackedSectorKey::pack (tk-symmetry/src/sector_key.rs:31-46).
uint64_t key_pack(int kind, const Qn* qns, int rank);
void key_unpack(int kind, uint64_t key, int rank, Qn* qns);

// QIndex (tk-symmetry/src/sector_key.rs:96-148), owned copy.
struct QIndex {
    std::vector<Qn> q;
    std::vector<int64_t> dim;
    std::vector<int64_t> off;
    int64_t total = 0;
    int find(const Qn& x) const;  // sector index or -1 (offset_of / dim_of)
    bool same_as(const QIndex& o) const;
    int n() const { return (int)q.size(); }
};
// Copies a tk_qindex; checks sectors are strictly sorted with positive dims.
bool qindex_from_abi(int kind, const tk_qindex& in, QIndex& out, std::string& err);

// Rank-4 MPO site tensor (s_in, s_out, w_L, w_R) read from the ABI.
struct Bst4 {
    int kind = 0;
    QIndex legs[4];
    std::vector<uint64_t> keys;
    std::vector<int64_t> offs;
    const double* data = nullptr;
};
bool bst4_from_abi(const tk_bst& t, Bst4& o, const char* name, std::string& err);
// Dense (d, d, wl, wr) copy in global indices (host data only).
bool mpo_dense(const Bst4& w, std::vector<double>& out, std::string& err);

// ---------------------------------------------------------------------------
// Sector-GEMM tables.  One launch of the grouped GEMM kernel walks a tile
// list; each tile belongs to a task (one output block) whose K dimension is a
// list of segments (one per contributing sector pair), so contributions to
// one output block are summed in registers without atomics.
//   A(i,k) = A[a_off + i*a_rs + k*a_cs],  B(k,j) = B[b_off + k*b_rs + j*b_cs]
//   C(i,j) = alpha * sum_seg A*B + beta * C   (C not read when beta == 0)
// ---------------------------------------------------------------------------
struct GemmSeg {
    int64_t a_off, b_off;
    int32_t a_rs, a_cs, b_rs, b_cs;
    int32_t K, pad;
};
struct GemmTask {
    int64_t c_off;
    int32_t c_rs, c_cs;
    int32_t M, N;
    int32_t seg_begin, seg_end;
    double alpha, beta;
};
// A tile is a square of edge 64 >> cls (cls 0: 64, 1: 32, 2: 16), chosen per
// task so small sector blocks are not padded to 64 x 64.
struct GemmTile {
    int32_t task, m0, n0, cls;
};
constexpr int kGemmTileClasses = 3;
// Channel combine (W_i*W_j applied between the two GEMM stages):
//   out[out_off + r*out_rs + c] = sum_t coef_t * in[in_off_t + r*in_rs_t + c]
struct CombJob {
    int64_t out_off;
    int32_t out_rs, rows, cols, term_begin, term_end, pad;
};
struct CombTerm {
    int64_t in_off;
    int32_t in_rs, pad;
    double coef;
};

// Host description of one dense<->flat sub-block copy (one state pair).
struct SubMap {
    int64_t dense_off, flat_off;
    int32_t rows, cols;  // rows = D_A (dense row stride D_R), cols = D_B
};

struct GemmTable {
    std::vector<GemmTask> tasks;
    std::vector<GemmSeg> segs;
    std::vector<GemmTile> tiles;
    double flops = 0.0;
};
// Tile class of an M x N task: the edge (64, 32 or 16) with the least
// padded area plus a fixed per-tile share.
int gemm_tile_class(int M, int N);
// Appends the output tiles of task `task_id`; with tile_m = tile_n = 64 the
// edge comes from gemm_tile_class, otherwise 64 x 64 tiles.
void gemm_add_tiles(GemmTable& g, int task_id, int tile_m, int tile_n);
// Orders tiles heaviest first (rows x cols x total K), stable.
void gemm_lpt_order(GemmTable& g, int tile_m, int tile_n);
// Every operand and output access of a table checked against buffer sizes.
bool gemm_table_ok(const GemmTable& g, int64_t na, int64_t nb, int64_t nc, const char* name, std::string& err);
bool comb_table_ok(const std::vector<CombJob>& jobs, const std::vector<CombTerm>& terms, int64_t n_in, int64_t n_out,
                   std::string& err);

// ---------------------------------------------------------------------------
// Split-precision (tensor-core) tables.  Both GEMM stages are regrouped into
// "stacks" that share one operand:
//   stage 1, one stack per ket sector A of L: rows = every L slab (A', ws, A)
//     stacked, columns = every psi sub-block (p, A, B) side by side, K = D_A
//     (stacks of at most TcOptions::tall_max_mtiles row tiles read and split the psi
//     operand straight from the fp64 vector inside the stage-1 kernel,
//     through the per-column tables xsrc / xstride; taller stacks, whose
//     row tiles would each split the same columns again, take it from a
//     bf16 hi/lo copy made once per matvec by the split kernel);
//   stage 3, one stack per bra sector B' of R: rows = every y sub-block
//     (p', A', B') stacked, columns = D_B', K = every R slab (B', ws, B)
//     concatenated.
// Operands are bf16 (hi, lo) pairs stored K-major in 64-element chunks: a
// stack's chunk c occupies `cstride` consecutive rows of 64 bf16 starting at
// row base + c*cstride, so one 2D TMA tensor map covers a whole buffer.
// K beyond a stack's extent is zero in both operands.
// ---------------------------------------------------------------------------
constexpr int kTcBM = 128;  // rows per tensor-core tile (UMMA M)
constexpr int kTcBN = 64;   // columns per tensor-core tile (UMMA N)
constexpr int kTcBK = 64;   // K chunk (128 bytes of bf16: one swizzle atom)

struct TcTile {
    int32_t a_row, a_cs;     // A operand row of chunk 0 at this tile's m0; rows between chunks
    int32_t b_row, b_cs;     // B operand row of chunk 0 at this tile's n0; rows between chunks
    int32_t kch, m_valid, n_valid, mode;  // mode 1: fp64 out through a row table; 2: fp32 out through column tables
    int64_t out_off;         // mode 1: row-table index of m0; mode 2: column-table index of n0
    int32_t ldc, n0;         // mode 1: n0 = column offset added to the row table; mode 2: ldc = m0
    int32_t n_mma, k_valid;  // UMMA N (n_valid rounded up to 16, <= kTcBN); stage 1: K of the stack (D_A)
    int32_t fill0, pad_;     // fused stage 3: chunk c's fill segments are fill_segs[fill_chunk[fill0 + c] ..)
};
// Fused stage 3 (the W_i W_j combine inside the stage-3 GEMM): a stage-3
// stack of at most TcOptions::fuse_max_ntiles column tiles builds its A
// operand (T2) chunk by chunk in shared memory from T1 instead of reading a
// T2 written by the combine kernel.  One fill segment = one rectangle of a
// chunk, element (r, k) = sum_t coef_t * T1[in_off_t + r * in_rs_t + k],
// written to tile row r0 + r, chunk column k0 + k (terms in
// TcTables::fill_terms, their in_off at the segment's first element).
struct TcFillSeg {
    int16_t r0, rows;   // tile rows [r0, r0 + rows), r0 + rows <= kTcBM
    int16_t k0, cols;   // chunk columns [k0, k0 + cols), k0 + cols <= kTcBK
    int32_t term_begin, term_end;
};
// psi sub-block -> stage-1 B operand of a tall stack (K-major chunks), hi/lo
// split.  One job = one 64 (a) x 32 (b) tile of a D_A x D_B sub-block, a0 a
// multiple of 64 (one K chunk).
struct TcSplitJob {
    int64_t src;             // flat offset of the (D_A x D_B) sub-block
    int32_t rows, cols;      // D_A (becomes K), D_B (becomes N)
    int32_t xrow, cstride;   // operand row of chunk 0 for column 0; rows between chunks
    int32_t a0, b0;          // tile origin inside the sub-block
};
// T1 (fp32) -> stage-3 A operand (K-major chunks), hi/lo split.  One job =
// rows [r0, r0 + rows) of one output slab, at most kTcCombMaxElems elements
// (one CTA each).  A job with at most kTcCombInline terms carries them in
// its descriptor as well (no second dependent table read).
struct TcCombTerm {
    int64_t in_off;
    int32_t in_rs;
    float coef;
};
constexpr int kTcCombInline = 2;
struct TcCombJob {
    int32_t t2row, cstride;  // operand row of chunk 0 for slab row 0; rows between chunks
    int32_t k0, rows, cols, term_begin, term_end, r0;
    TcCombTerm inl[kTcCombInline];  // terms[term_begin .. term_end) when there are at most kTcCombInline
};
constexpr int kTcCombMaxElems = 512;
constexpr int kTcPsiPieces = 8;
struct TcTables {
    int64_t lq_rows = 0, rq_rows = 0, xq_rows = 0, t2q_rows = 0, t1_total = 0;
    std::vector<uint16_t> lq_hi, lq_lo, rq_hi, rq_lo;  // constant operands, split at plan time
    std::vector<double> lq64, rq64;                    // the same stacks in FP64 (stacked FP64 schedule)
    std::vector<double> lq64_im, rq64_im;              // their imaginary parts (complex environments)
    std::vector<double> term_coef64;                   // FP64 coefficients of `terms`
    std::vector<TcTile> tiles1, tiles3;
    std::vector<TcTile> tiles1x;       // stage-1 tiles of tall stacks (B operand from the split copy)
    // psi in kTcPsiPieces pieces at block boundaries x_cut[0] = 0 < ... <
    // x_cut[kTcPsiPieces] = |psi|: tiles1[n1_cut[j], n1_cut[j + 1]) read psi
    // only below x_cut[j + 1] (a host-buffer matvec starts them once that much
    // of psi is on the device)
    int32_t n1_cut[kTcPsiPieces + 1] = {};
    int64_t x_cut[kTcPsiPieces + 1] = {};
    std::vector<TcSplitJob> split;     // psi -> split copy, tall stacks only
    std::vector<TcCombJob> jobs;
    std::vector<TcCombTerm> terms;
    // fused stage 3: tiles (mode 3), their per-chunk segment ranges and segments
    std::vector<TcTile> tiles3f;
    std::vector<int32_t> fill_chunk;   // per fused tile: kch + 1 offsets into fill_segs
    std::vector<TcFillSeg> fill_segs;
    std::vector<TcCombTerm> fill_terms;
    double fill_term_elems = 0.0;      // sum over fill segments of elements x terms (T1 reads)
    std::vector<int64_t> yrow;  // y element offset of every stage-3 operand row
    // T1 is stored per (stack A, column block (p, B)) as a row-major
    // [rows_A x D_B] matrix: element (r, c) of stack A sits at
    // t1col_base[c] + r * t1col_stride[c] (c = global stage-1 column).
    std::vector<int64_t> t1col_base;
    std::vector<int32_t> t1col_stride;
    // stage-1 B operand: column c is psi[xsrc[c] + k * xstride[c]], k < K of its stack
    std::vector<int64_t> xsrc;
    std::vector<int32_t> xstride;
    double mma_flops = 0.0;     // padded tensor-core work of both stages (one product)
    int32_t max_kch1 = 0, max_kch1x = 0, max_kch3 = 0, max_kch3f = 0;
};

// Schedule options of the split-precision tables (the autotuner's knobs):
//   tall_max_mtiles: stage-1 stacks of at most this many 128-row tiles split
//     psi inside the GEMM kernel; taller ones take a split copy made once per
//     matvec (every row tile would otherwise split the same columns again);
//   fuse_max_ntiles: stage-3 stacks of at most this many column tiles run the
//     W_i W_j combine inside the GEMM kernel (0: never; each column tile
//     rebuilds the operand, so only narrow stacks qualify).
//   combine_warps: the separate combine as one CTA per job (0), persistent
//     warps that prefetch their next job (1), one warp per job (2), or one
//     64-thread CTA per job, eight elements per thread (3).
//   stage1_persistent: the in-kernel-split stage 1 as a persistent,
//     warp-specialised kernel (1) or one CTA per tile (0).
//   stage1_narrow: the one-CTA-per-tile stage 1 in 32-wide K chunks with a
//     single 24 KB stage, eight CTAs per SM (1), or 64-wide chunks, four CTAs
//     per SM (0); the same MMAs in the same order either way.
struct TcOptions {
    int32_t tall_max_mtiles = 3;
    int32_t fuse_max_ntiles = 0;
    int32_t combine_warps = 0;
    int32_t stage1_persistent = 0;
    int32_t stage1_narrow = 0;
};

// The sector structure the split-precision tables are built from, kept with
// the host tables so that a plan can rebuild them with other options.
struct TcSource {
    struct Term {
        int64_t p, wl;
        double c;
    };
    int nA = 0, nB = 0, nWL = 0, nWR = 0;
    int64_t P = 0, nwr = 0;
    QIndex QA, QB, WL, WR;
    std::vector<int64_t> lblk, rblk, sub;  // slab / two-site sub-block offsets (-1: absent)
    std::vector<std::vector<Term>> byout;  // W_ij terms by (p', w_R)
    std::vector<int> wl_sec;
    std::vector<int64_t> wl_loc;
};

// Everything the device needs for one two-site H_eff, built on the host.
struct Heff2Tables {
    int kind = 0;
    int64_t d_i = 0, d_j = 0, d_l = 0, d_r = 0, nwl = 0, nwr = 0;
    // two-site block layout (FlatBlockStorage order: ascending packed key)
    std::vector<uint64_t> keys;
    std::vector<int64_t> blk_off;
    int64_t total = 0;
    std::vector<SubMap> submaps;
    // non-zero sector slabs of L ([(a',w)][a]) and R ([b'][(w,b)])
    std::vector<double> lbuf, rbuf;
    // stage 1: T1 = L * psi ; stage 2: T2 = W_ij (x) T1 ; stage 3: y = T2 * R^T
    GemmTable g1, g3;
    std::vector<CombJob> jobs;
    std::vector<CombTerm> terms;
    int64_t t1_total = 0, t2_total = 0;
    double comb_flops = 0.0;
    double alg_bytes = 0.0;
    int64_t n_wij_terms = 0;
    // split-precision (tensor-core) regrouping of the same work
    TcTables tc;
    bool tc_built = false;  // tc holds the tables of tcopt (built on first use)
    TcOptions tcopt;
    std::shared_ptr<TcSource> tcsrc;
    // the stacked FP64 schedule's tables (the split stacks in FP64; built on demand)
    TcTables f64st;
};
// Builds T.f64st: the stack tables with every stage-1 column read through
// its psi table and no fused stage 3, the operand stacks in FP64 (and, for
// complex environments, their imaginary parts from host copies of the
// imaginary slab arrays, laid out like T.lbuf / T.rbuf).
tk_status build_f64_stacks(Heff2Tables& T, std::string& err, const double* lbuf_im = nullptr,
                           const double* rbuf_im = nullptr);
// Builds T.tc with T.tcopt unless built already (the split tables of a plan
// that never runs split precision are never built).
tk_status ensure_tc_tables(Heff2Tables& T, std::string& err);
// Rebuilds T.tc with options `o` (T.tc and T.tcopt unchanged on failure).
tk_status rebuild_tc_tables(Heff2Tables& T, const TcOptions& o, std::string& err);

// bf16 bit pattern of a float, round to nearest even (NaN kept quiet).
uint16_t f32_to_bf16_bits(float f);
float bf16_bits_to_f32(uint16_t b);

// Host-allocation checkpoint of the table builders: throws std::bad_alloc
// at the countdown-th checkpoint once tk_debug_fail_host_alloc armed one
// (test hook for the TK_ERR_OOM paths; a no-op otherwise).
void host_alloc_checkpoint();

// Runs a host table builder and turns a C++ exception (a failed host
// allocation above all) into a status code with `err` set: no exception may
// cross the C ABI.
template <class F>
tk_status guard_host(const char* what, std::string& err, F&& build) {
    try {
        return build();
    } catch (const std::bad_alloc&) {
        err = std::string(what) + ": host allocation failed";
        return TK_ERR_OOM;
    } catch (const std::length_error&) {
        err = std::string(what) + ": host tables too large";
        return TK_ERR_OOM;
    } catch (const std::exception& e) {
        err = std::string(what) + ": " + e.what();
        return TK_ERR_INVALID_ARG;
    }
}

// Builds the tables; returns TK_OK or an error code with `err` set.  With
// l_blocks / r_blocks (host copies of environments in the canonical block
// layout of env_layout) the environments' dense data are not read.
tk_status build_heff2_tables(const tk_env& L, const tk_env& R, const tk_bst& wi, const tk_bst& wj,
                             const int32_t* psi_flux, int tile_m, int tile_n, Heff2Tables& out,
                             std::string& err, const double* l_blocks = nullptr, const double* r_blocks = nullptr);

// Canonical block layout of a block-sparse environment (bra, mpo, ket): every
// sector triple with q(bra) = q(ket) + q(mpo), ascending packed key (bra in
// the low bits), blocks back to back, each row-major (a', w, a).
struct EnvLayout {
    std::vector<std::array<int, 3>> tri;  // (bra sector, mpo sector, ket sector)
    std::vector<uint64_t> keys;
    std::vector<int64_t> off;             // block offsets
    int64_t total = 0;
};
void env_layout(int kind, const QIndex& bra, const QIndex& mpo, const QIndex& ket, EnvLayout& out);

// Thread-local last-error message.
void set_error(const std::string& msg);
// The context's scratch (abi.cu): device arena and page-locked staging of at
// least `bytes` (grown by half again when too small, contents not kept), and
// its stream (created on first use).  Return TK_OK or a status with the
// message set.
tk_status ctx_dev_scratch(tk_ctx* ctx, size_t bytes, void** out);
tk_status ctx_host_stage(tk_ctx* ctx, size_t bytes, void** out);
tk_status ctx_stream(tk_ctx* ctx, void** out);
// Packs host arrays back to back (256-byte aligned) for one host-to-device copy.
struct Blob {
    // The pieces of one host-to-device transfer: each piece is recorded with
    // its source, and copy_to() copies every source once, straight into the
    // page-locked staging buffer (the sources must outlive that call).
    struct Ref {
        size_t at;
        const void* p;
        size_t n;
    };
    std::vector<Ref> refs;
    size_t end = 0;   // end of the transferred bytes
    size_t tail = 0;  // end of the reserved space past them (written on the device)
    size_t add(const void* p, size_t n) {
        const size_t at = (end + 255) & ~(size_t)255;
        if (n) refs.push_back({at, p, n});
        end = at + n;
        return at;
    }
    size_t reserve(size_t n) {  // space without data (written on the device)
        const size_t at = (end + 255) & ~(size_t)255;
        end = at;
        tail = at + n;
        return at;
    }
    size_t size() const { return end; }
    size_t device_size() const { return std::max(end, tail); }
    void copy_to(void* dst) const {
        unsigned char* d = static_cast<unsigned char*>(dst);
        for (const Ref& r : refs) std::memcpy(d + r.at, r.p, r.n);
    }
};
// Releases the context's cuSOLVER handle (dense.cu).
void ctx_release_solver(tk_ctx* ctx);

}  // namespace tk
