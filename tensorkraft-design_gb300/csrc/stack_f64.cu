// stack_f64.cu -- the FP64 matvec on operand stacks (TK_SCHED_STACKED).
//
// The grouped FP64 schedule runs one GEMM task per output sector block; with
// sector dimensions around 13 and one or two MPO channels per slab, most of
// its tasks are a few rows tall and a square tile covers them sparsely (about
// 60 % of the FP64 FMAs it issues are useful on Hubbard D=2048).  This
// schedule regroups the same work the way the split-precision path does
// (TcTables, built with every psi column read through its table and no
// fused stage 3):
//   stage 1, one stack per ket sector A of L: T1 = L_stack(A) * psi_A, the
//     stack's rows every L slab (A', w, A), its columns every psi sub-block
//     (p, A, B), K = D_A;
//   combine: T2 = sum coef * T1 over the W_i W_j terms, written in the
//     stage-3 operand layout (K-major 64-wide chunks, zero padding);
//   stage 3, one stack per bra sector B' of R: y = T2_stack * R_stack^T
//     through the y row table.
// The operands are the split path's stacks in FP64; the GEMMs run on the
// FP64 pipe (this GPU's FP64 tensor rate is no higher than its CUDA-core
// FP64 rate).  On this GPU an FP64 FMA occupies its pipe some thirty times
// longer than any other instruction a thread runs, so the kernels are laid
// out to issue as few FP64 FMAs as possible, index arithmetic being free
// next to them:
//   - a piece (the work of one CTA) is at most 32 x 64 outputs, laid densely
//     over the 256 threads (DenseMap);
//   - k steps over the piece's K segments only: stage 1 the stack's true K,
//     stage 3 the column ranges of T2 that its rows hold (the combine leaves
//     the rest of a T2 stack zero: the W_i W_j channels that do not reach
//     those rows), with no predicated-off FMA past a segment's end;
//   - pieces are cut so that each holds at most a share of the stage's
//     FMAs, and go out longest first.
// Every output sums its k in ascending order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <set>
#include <string>

#include "tk_plan.cuh"

namespace tk {
namespace {

constexpr int SBN = kTcBN;  // 64 columns per piece (the stacks' column tiles)
constexpr int SBK = 16;     // k step through shared memory
constexpr int ST = 256;
constexpr int SBM = 32;     // rows per piece at most
constexpr int RPT = SBM * SBN / ST;  // outputs per thread of a full piece

// One CTA's work: rows [a_row, a_row + m_valid) (operand rows of chunk 0) of
// a stack against n_valid columns, over the K segments segs[seg0, seg0 + nseg).
struct F64Piece {
    int32_t a_row, a_cs, b_row, b_cs;
    int32_t m_valid, n_valid;
    int32_t ldc, n0;   // stage 1: T1 row of the first row; stage 3: y column offset
    int64_t out_off;   // stage 1: column-table index of column 0; stage 3: y row-table index of row 0
    int32_t seg0, nseg;
};
struct KSeg {
    int32_t kb, ke;  // k in [kb, ke)
};

// The outputs of a piece lie densely over the threads: output e (row e / nv,
// column e % nv of the m_valid x nv block) belongs to thread e % ST, its
// round e / ST.  A warp runs only the rounds that hold one of its outputs,
// so the FMAs it issues are the piece's outputs times K, rounded up to whole
// warps.
struct DenseMap {
    int nv, total, rounds;  // columns, outputs, rounds of this warp
    __device__ DenseMap(int m_valid, int n_valid, int warp) : nv(n_valid), total(m_valid * n_valid) {
        rounds = total > 32 * warp ? (total - 32 * warp + ST - 1) / ST : 0;
    }
};

// acc[r] += sum over k < kl of A[k][m_r] * B[k][n_r], k ascending; complex
// (CPLX): (ar + i ai)(br + i bi) accumulated as re += ar br - ai bi and
// im += ar bi + ai br.  A full step is unrolled; a short one loops exactly kl
// times, so that no FMA past the segment's end is issued (predicated off, it
// would still hold the pipe).
template <bool CPLX>
__device__ __forceinline__ void dense_kstep(const double (*Ar)[SBM + 1], const double (*Ai)[SBM + 1],
                                            const double (*Br)[SBN + 1], const double (*Bi)[SBN + 1], int kl,
                                            const DenseMap& d, int tid, double* accr, double* acci) {
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
        if (r < d.rounds) {
            const int e = min(tid + ST * r, d.total - 1);  // lanes past the end read a valid element
            const int m = e / d.nv, n = e - m * d.nv;
            double sr = accr[r], si = CPLX ? acci[r] : 0.0;
            auto step = [&](int k) {
                sr = fma(Ar[k][m], Br[k][n], sr);
                if constexpr (CPLX) {
                    sr = fma(-Ai[k][m], Bi[k][n], sr);
                    si = fma(Ar[k][m], Bi[k][n], si);
                    si = fma(Ai[k][m], Br[k][n], si);
                }
            };
            if (kl == SBK) {
#pragma unroll
                for (int k = 0; k < SBK; ++k) step(k);
            } else {
#pragma unroll 1
                for (int k = 0; k < kl; ++k) step(k);
            }
            accr[r] = sr;
            if constexpr (CPLX) acci[r] = si;
        }
    }
}

// k in [k0, k0 + kl) of a stack operand (rows m < rows_valid of chunk-0 row
// `row`, `cs` rows between chunks) into S[k][m].
__device__ __forceinline__ void load_op_a(double (*S)[SBM + 1], const double* __restrict__ q, int32_t row, int32_t cs,
                                          int rows_valid, int k0, int kl, int tid) {
#pragma unroll
    for (int r = 0; r < SBM * SBK / ST; ++r) {
        const int e = tid + ST * r, k = e & 15, m = e >> 4, kk = k0 + k;
        double v = 0.0;
        if (m < rows_valid && k < kl) v = q[(((int64_t)row + (int64_t)(kk >> 6) * cs + m) << 6) + (kk & 63)];
        S[k][m] = v;
    }
}

__device__ __forceinline__ void load_op_b(double (*S)[SBN + 1], const double* __restrict__ q, int32_t row, int32_t cs,
                                          int rows_valid, int k0, int kl, int tid) {
#pragma unroll
    for (int r = 0; r < SBN * SBK / ST; ++r) {
        const int e = tid + ST * r, k = e & 15, n = e >> 4, kk = k0 + k;
        double v = 0.0;
        if (n < rows_valid && k < kl) v = q[(((int64_t)row + (int64_t)(kk >> 6) * cs + n) << 6) + (kk & 63)];
        S[k][n] = v;
    }
}

// Stage 1: T1 = L stacks * psi (CPLX: both complex, planar).
template <bool CPLX>
__global__ void __launch_bounds__(ST, 4) stack_gemm1_f64_kernel(const F64Piece* __restrict__ pieces,
                                                                const KSeg* __restrict__ segs,
                                                                const double* __restrict__ lq,
                                                                const double* __restrict__ lq_im,
                                                                const double* __restrict__ x,
                                                                const double* __restrict__ x_im,
                                                                const int64_t* __restrict__ xsrc,
                                                                const int32_t* __restrict__ xstride,
                                                                const int64_t* __restrict__ colbase,
                                                                const int32_t* __restrict__ colstride,
                                                                double* __restrict__ t1, double* __restrict__ t1_im) {
    __shared__ double Ar[SBK][SBM + 1], Br[SBK][SBN + 1];
    __shared__ double Ai[CPLX ? SBK : 1][SBM + 1], Bi[CPLX ? SBK : 1][SBN + 1];
    const F64Piece t = pieces[blockIdx.x];
    const int tid = threadIdx.x;
    const int ln = tid & 63;  // the B column this thread loads
    const bool lv = ln < t.n_valid;
    const int64_t src = lv ? xsrc[t.out_off + ln] : 0;
    const int32_t str = lv ? xstride[t.out_off + ln] : 0;
    const DenseMap d(t.m_valid, t.n_valid, tid >> 5);
    double accr[RPT], acci[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) accr[r] = acci[r] = 0.0;
    for (int sg = t.seg0; sg < t.seg0 + t.nseg; ++sg) {
        const KSeg g = segs[sg];
        for (int k0 = g.kb; k0 < g.ke; k0 += SBK) {
            const int kl = min(SBK, g.ke - k0);
            load_op_a(Ar, lq, t.a_row, t.a_cs, t.m_valid, k0, kl, tid);
            if constexpr (CPLX) load_op_a(Ai, lq_im, t.a_row, t.a_cs, t.m_valid, k0, kl, tid);
#pragma unroll
            for (int r = 0; r < SBN * SBK / ST; ++r) {
                const int k = (tid >> 6) + 4 * r, kk = k0 + k;
                const bool ok = lv && k < kl;
                Br[k][ln] = ok ? x[src + (int64_t)kk * str] : 0.0;
                if constexpr (CPLX) Bi[k][ln] = ok ? x_im[src + (int64_t)kk * str] : 0.0;
            }
            __syncthreads();
            dense_kstep<CPLX>(Ar, Ai, Br, Bi, kl, d, tid, accr, acci);
            __syncthreads();
        }
    }
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
        const int e = tid + ST * r;
        if (r < d.rounds && e < d.total) {
            const int m = e / d.nv, n = e - m * d.nv;
            const int64_t o = colbase[t.out_off + n] + (int64_t)(t.ldc + m) * colstride[t.out_off + n];
            t1[o] = accr[r];
            if constexpr (CPLX) t1_im[o] = acci[r];
        }
    }
}

// Stage 3: y = T2 stacks * R stacks^T (CPLX: both complex, planar).
template <bool CPLX>
__global__ void __launch_bounds__(ST, 4) stack_gemm3_f64_kernel(const F64Piece* __restrict__ pieces,
                                                                const KSeg* __restrict__ segs,
                                                                const double* __restrict__ t2,
                                                                const double* __restrict__ t2_im,
                                                                const double* __restrict__ rq,
                                                                const double* __restrict__ rq_im,
                                                                const int64_t* __restrict__ yrow,
                                                                double* __restrict__ y, double* __restrict__ y_im) {
    __shared__ double Ar[SBK][SBM + 1], Br[SBK][SBN + 1];
    __shared__ double Ai[CPLX ? SBK : 1][SBM + 1], Bi[CPLX ? SBK : 1][SBN + 1];
    const F64Piece t = pieces[blockIdx.x];
    const int tid = threadIdx.x;
    const DenseMap d(t.m_valid, t.n_valid, tid >> 5);
    double accr[RPT], acci[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) accr[r] = acci[r] = 0.0;
    for (int sg = t.seg0; sg < t.seg0 + t.nseg; ++sg) {
        const KSeg g = segs[sg];
        for (int k0 = g.kb; k0 < g.ke; k0 += SBK) {
            const int kl = min(SBK, g.ke - k0);
            load_op_a(Ar, t2, t.a_row, t.a_cs, t.m_valid, k0, kl, tid);
            load_op_b(Br, rq, t.b_row, t.b_cs, t.n_valid, k0, kl, tid);
            if constexpr (CPLX) {
                load_op_a(Ai, t2_im, t.a_row, t.a_cs, t.m_valid, k0, kl, tid);
                load_op_b(Bi, rq_im, t.b_row, t.b_cs, t.n_valid, k0, kl, tid);
            }
            __syncthreads();
            dense_kstep<CPLX>(Ar, Ai, Br, Bi, kl, d, tid, accr, acci);
            __syncthreads();
        }
    }
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
        const int e = tid + ST * r;
        if (r < d.rounds && e < d.total) {
            const int m = e / d.nv, n = e - m * d.nv;
            const int64_t o = yrow[t.out_off + m] + t.n0 + n;
            y[o] = accr[r];
            if constexpr (CPLX) y_im[o] = acci[r];
        }
    }
}

// T2 = sum coef * T1 for one combine job (rows r0 .. r0 + rows of a slab),
// written into the chunked stage-3 operand layout.
__global__ void __launch_bounds__(128) stack_combine_f64_kernel(const TcCombJob* __restrict__ jobs,
                                                                const TcCombTerm* __restrict__ terms,
                                                                const double* __restrict__ coef,
                                                                const double* __restrict__ t1,
                                                                double* __restrict__ t2) {
    const TcCombJob j = jobs[blockIdx.x];
    const int n = j.rows * j.cols;
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int rl = e / j.cols, c = e - rl * j.cols, r = j.r0 + rl;
        double acc = 0.0;
        for (int q = j.term_begin; q < j.term_end; ++q)
            acc = fma(coef[q], t1[terms[q].in_off + (int64_t)r * terms[q].in_rs + c], acc);
        const int k = j.k0 + c;
        t2[(((int64_t)j.t2row + (int64_t)(k >> 6) * j.cstride + r) << 6) + (k & 63)] = acc;
    }
}

double seg_len(const std::vector<KSeg>& segs, int32_t s0, int32_t n) {
    double k = 0.0;
    for (int32_t s = s0; s < s0 + n; ++s) k += segs[(size_t)s].ke - segs[(size_t)s].kb;
    return k;
}

// One run of rows [r_begin, r_end) of a 128-row stack tile that share the K
// segments segs[seg0, seg0 + nseg): cut into pieces of at most SBM rows, and
// more where a piece would exceed `target` FMAs (down to one row).  A piece
// is the tile with its first row moved: stage 1 (mode 2) shifts the operand
// row and the T1 row (ldc), stage 3 (mode 1) the operand row and the y
// row-table index.
void cut_run(const TcTile& t, int r_begin, int r_end, int32_t seg0, int32_t nseg, double klen, double target,
             std::vector<F64Piece>& out) {
    const int R = r_end - r_begin;
    const double cost = (double)R * t.n_valid * klen;
    const int64_t want = std::max<int64_t>((R + SBM - 1) / SBM, (int64_t)std::ceil(cost / target));
    const int pieces = (int)std::min<int64_t>(want, R);
    const int rows = (R + pieces - 1) / pieces;
    for (int r0 = r_begin; r0 < r_end; r0 += rows) {
        F64Piece p;
        p.a_row = t.a_row + r0;
        p.a_cs = t.a_cs;
        p.b_row = t.b_row;
        p.b_cs = t.b_cs;
        p.m_valid = std::min(rows, r_end - r0);
        p.n_valid = t.n_valid;
        p.ldc = t.mode == 2 ? t.ldc + r0 : t.ldc;
        p.n0 = t.n0;
        p.out_off = t.mode == 2 ? t.out_off : t.out_off + r0;
        p.seg0 = seg0;
        p.nseg = nseg;
        out.push_back(p);
    }
}

void sort_longest_first(std::vector<F64Piece>& v, const std::vector<KSeg>& segs) {
    std::vector<std::pair<double, size_t>> c(v.size());
    for (size_t i = 0; i < v.size(); ++i)
        c[i] = {-(double)v[i].m_valid * v[i].n_valid * seg_len(segs, v[i].seg0, v[i].nseg), i};
    std::stable_sort(c.begin(), c.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    std::vector<F64Piece> o(v.size());
    for (size_t i = 0; i < v.size(); ++i) o[i] = v[c[i].second];
    v.swap(o);
}

// Stage 1: every row of a stack needs all of its K = D_A.
void stage1_pieces(const std::vector<TcTile>& tiles, std::vector<F64Piece>& out, std::vector<KSeg>& segs) {
    double total = 0.0;
    for (const TcTile& t : tiles) total += (double)t.m_valid * t.n_valid * t.k_valid;
    const double target = std::max(1.0, total / (152.0 * 16.0));
    for (const TcTile& t : tiles) {
        const int32_t s0 = (int32_t)segs.size();
        segs.push_back({0, t.k_valid});
        cut_run(t, 0, t.m_valid, s0, 1, t.k_valid, target, out);
    }
    sort_longest_first(out, segs);
}

// Stage 3: row r of a T2 stack holds the columns the combine jobs write to
// it (each job one rectangle of rows and K columns); a run of consecutive
// rows with the same merged column ranges becomes pieces over those ranges.
bool stage3_pieces(const TcTables& C, std::vector<F64Piece>& out, std::vector<KSeg>& segs, std::string& err) {
    // column ranges per operand row of chunk 0 (the rows tiles and jobs index)
    std::vector<std::vector<KSeg>> rowk((size_t)std::max<int64_t>(C.t2q_rows, 0));
    for (const TcCombJob& j : C.jobs)
        for (int r = j.r0; r < j.r0 + j.rows; ++r) rowk[(size_t)j.t2row + r].push_back({j.k0, j.k0 + j.cols});
    for (std::vector<KSeg>& v : rowk) {
        if (v.empty()) continue;
        std::sort(v.begin(), v.end(), [](const KSeg& a, const KSeg& b) { return a.kb < b.kb; });
        std::vector<KSeg> m;
        for (const KSeg& g : v) {
            if (!m.empty() && g.kb <= m.back().ke)
                m.back().ke = std::max(m.back().ke, g.ke);
            else
                m.push_back(g);
        }
        v.swap(m);
    }
    auto klen = [](const std::vector<KSeg>& v) {
        double k = 0.0;
        for (const KSeg& g : v) k += g.ke - g.kb;
        return k;
    };
    auto same = [](const std::vector<KSeg>& a, const std::vector<KSeg>& b) {
        if (a.size() != b.size()) return false;
        for (size_t i = 0; i < a.size(); ++i)
            if (a[i].kb != b[i].kb || a[i].ke != b[i].ke) return false;
        return true;
    };
    double total = 0.0;
    for (const TcTile& t : C.tiles3)
        for (int m = 0; m < t.m_valid; ++m) total += (double)t.n_valid * klen(rowk[(size_t)t.a_row + m]);
    const double target = std::max(1.0, total / (152.0 * 16.0));
    for (const TcTile& t : C.tiles3) {
        int m = 0;
        while (m < t.m_valid) {
            const std::vector<KSeg>& ks = rowk[(size_t)t.a_row + m];
            if (!ks.empty() && (ks.front().kb < 0 || ks.back().ke > t.k_valid)) {
                err = "stacked FP64 stage-3 row reaches past its stack's K";
                return false;
            }
            int e = m + 1;
            while (e < t.m_valid && same(rowk[(size_t)t.a_row + e], ks)) ++e;
            // rows no combine job writes get a piece without segments: it stores zeros
            const int32_t s0 = (int32_t)segs.size();
            segs.insert(segs.end(), ks.begin(), ks.end());
            cut_run(t, m, e, s0, (int32_t)ks.size(), klen(ks), target, out);
            m = e;
        }
    }
    sort_longest_first(out, segs);
    return true;
}

}  // namespace

struct F64Stack {
    DevBuf<double> lq, rq, t1, t2, coef;
    DevBuf<double> lq_im, rq_im, t1_im, t2_im;  // complex environments only
    bool cplx = false;
    DevBuf<F64Piece> pieces1, pieces3;
    DevBuf<KSeg> segs;
    DevBuf<TcCombJob> jobs;
    DevBuf<TcCombTerm> terms;
    DevBuf<int64_t> yrow, colbase, xsrc;
    DevBuf<int32_t> colstride, xstride;
    int n1 = 0, n3 = 0, njobs = 0;
    double bytes[3] = {0.0, 0.0, 0.0};  // per stage, without the psi / y vectors
};

void F64StackDeleter::operator()(F64Stack* p) const { delete p; }

tk_status f64stack_create(const TcTables& C, std::unique_ptr<F64Stack, F64StackDeleter>& out, std::string& err) {
    if (!C.tiles1x.empty() || !C.tiles3f.empty()) {
        err = "stacked FP64 tables with split-copy or fused tiles";
        return TK_ERR_INVALID_ARG;
    }
    for (const std::vector<TcTile>* v : {&C.tiles1, &C.tiles3})
        for (const TcTile& t : *v)
            if (t.m_valid <= 0 || t.m_valid > kTcBM || t.n_valid <= 0 || t.n_valid > SBN) {
                err = "stacked FP64 tile shape";
                return TK_ERR_INVALID_ARG;
            }
    std::vector<KSeg> segs;
    std::vector<F64Piece> p1, p3;
    stage1_pieces(C.tiles1, p1, segs);
    if (!stage3_pieces(C, p3, segs, err)) return TK_ERR_INVALID_ARG;
    std::unique_ptr<F64Stack, F64StackDeleter> p(new F64Stack);
    cudaError_t e = cudaSuccess;
    if ((e = p->lq.upload(C.lq64)) != cudaSuccess || (e = p->rq.upload(C.rq64)) != cudaSuccess ||
        (e = p->pieces1.upload(p1)) != cudaSuccess || (e = p->pieces3.upload(p3)) != cudaSuccess ||
        (e = p->segs.upload(segs)) != cudaSuccess ||
        (e = p->jobs.upload(C.jobs)) != cudaSuccess || (e = p->terms.upload(C.terms)) != cudaSuccess ||
        (e = p->coef.upload(C.term_coef64)) != cudaSuccess || (e = p->yrow.upload(C.yrow)) != cudaSuccess ||
        (e = p->colbase.upload(C.t1col_base)) != cudaSuccess || (e = p->colstride.upload(C.t1col_stride)) != cudaSuccess ||
        (e = p->xsrc.upload(C.xsrc)) != cudaSuccess || (e = p->xstride.upload(C.xstride)) != cudaSuccess ||
        (e = p->t1.alloc((size_t)std::max<int64_t>(C.t1_total, 1))) != cudaSuccess ||
        (e = p->t2.alloc((size_t)std::max<int64_t>(C.t2q_rows * kTcBK, 1))) != cudaSuccess ||
        (e = cudaMemset(p->t2.p, 0, sizeof(double) * p->t2.n)) != cudaSuccess) {
        err = std::string("stacked FP64 operands: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? TK_ERR_OOM : TK_ERR_CUDA;
    }
    p->cplx = !C.lq64_im.empty() || !C.rq64_im.empty();
    if (p->cplx &&
        ((e = p->lq_im.upload(C.lq64_im)) != cudaSuccess || (e = p->rq_im.upload(C.rq64_im)) != cudaSuccess ||
         (e = p->t1_im.alloc(p->t1.n)) != cudaSuccess || (e = p->t2_im.alloc(p->t2.n)) != cudaSuccess ||
         (e = cudaMemset(p->t2_im.p, 0, sizeof(double) * p->t2_im.n)) != cudaSuccess)) {
        err = std::string("stacked FP64 imaginary operands: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? TK_ERR_OOM : TK_ERR_CUDA;
    }
    if (p->cplx && (C.lq64_im.size() != C.lq64.size() || C.rq64_im.size() != C.rq64.size())) {
        err = "stacked FP64 imaginary stacks of another size";
        return TK_ERR_INVALID_ARG;
    }
    // Bytes each stage must move at least: every stack element a piece reads
    // once (rows read by several column tiles count once), T1 written / read
    // once, T2 written / read once.
    auto stack_elems = [&](const std::vector<F64Piece>& v, bool a_side) {
        std::set<std::pair<int32_t, int32_t>> seen;
        double n = 0.0;
        for (const F64Piece& q : v)
            if (seen.insert({a_side ? q.a_row : q.b_row, a_side ? q.m_valid : q.n_valid}).second)
                n += (double)(a_side ? q.m_valid : q.n_valid) * seg_len(segs, q.seg0, q.nseg);
        return n;
    };
    double comb_reads = 0.0;
    for (const TcCombJob& j : C.jobs) comb_reads += (double)j.rows * j.cols * (j.term_end - j.term_begin);
    const double t2_elems = stack_elems(p3, true);
    p->bytes[0] = 8.0 * (stack_elems(p1, true) + (double)C.t1_total);
    p->bytes[1] = 8.0 * (std::min<double>((double)C.t1_total, comb_reads) + t2_elems);
    p->bytes[2] = 8.0 * (t2_elems + stack_elems(p3, false));
    p->n1 = (int)p1.size();
    p->n3 = (int)p3.size();
    p->njobs = (int)C.jobs.size();
    out = std::move(p);
    return TK_OK;
}

cudaError_t f64stack_stage(F64Stack& p, const double* x, double* y, cudaStream_t s, int stage) {
    if (stage == 0 && p.n1 > 0)
        stack_gemm1_f64_kernel<false><<<p.n1, ST, 0, s>>>(p.pieces1.p, p.segs.p, p.lq.p, nullptr, x, nullptr,
                                                          p.xsrc.p, p.xstride.p, p.colbase.p, p.colstride.p, p.t1.p,
                                                          nullptr);
    else if (stage == 1 && p.njobs > 0)
        stack_combine_f64_kernel<<<p.njobs, 128, 0, s>>>(p.jobs.p, p.terms.p, p.coef.p, p.t1.p, p.t2.p);
    else if (stage == 2 && p.n3 > 0)
        stack_gemm3_f64_kernel<false><<<p.n3, ST, 0, s>>>(p.pieces3.p, p.segs.p, p.t2.p, nullptr, p.rq.p, nullptr,
                                                          p.yrow.p, y, nullptr);
    return cudaGetLastError();
}

cudaError_t f64stack_apply(F64Stack& p, const double* x, double* y, cudaStream_t s) {
    for (int stage = 0; stage < 3; ++stage) {
        cudaError_t e = f64stack_stage(p, x, y, s, stage);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t f64stack_apply_complex(F64Stack& p, const double* xr, const double* xi, double* yr, double* yi,
                                   cudaStream_t s) {
    if (!p.cplx) return cudaErrorInvalidValue;
    if (p.n1 > 0)
        stack_gemm1_f64_kernel<true><<<p.n1, ST, 0, s>>>(p.pieces1.p, p.segs.p, p.lq.p, p.lq_im.p, xr, xi, p.xsrc.p,
                                                         p.xstride.p, p.colbase.p, p.colstride.p, p.t1.p, p.t1_im.p);
    if (p.njobs > 0) {
        // the W_i W_j coefficients are real: the combine acts on each part
        stack_combine_f64_kernel<<<p.njobs, 128, 0, s>>>(p.jobs.p, p.terms.p, p.coef.p, p.t1.p, p.t2.p);
        stack_combine_f64_kernel<<<p.njobs, 128, 0, s>>>(p.jobs.p, p.terms.p, p.coef.p, p.t1_im.p, p.t2_im.p);
    }
    if (p.n3 > 0)
        stack_gemm3_f64_kernel<true><<<p.n3, ST, 0, s>>>(p.pieces3.p, p.segs.p, p.t2.p, p.t2_im.p, p.rq.p, p.rq_im.p,
                                                         p.yrow.p, yr, yi);
    return cudaGetLastError();
}

int f64stack_launches(const F64Stack& p) { return (p.n1 > 0) + (p.njobs > 0) + (p.n3 > 0); }

void f64stack_bytes(const F64Stack& p, double out[3]) {
    for (int i = 0; i < 3; ++i) out[i] = p.bytes[i];
}

}  // namespace tk
