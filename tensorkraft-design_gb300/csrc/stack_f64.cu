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
// FP64 rate) in 128 x 64 tiles of 256 threads, 8 x 4 outputs per thread,
// k stepping over the stack's true K only and each warp skipping the row
// groups past the tile's valid rows.  Every output sums k in ascending order.
#include <cuda_runtime.h>

#include <algorithm>
#include <set>
#include <string>

#include "tk_plan.cuh"

namespace tk {
namespace {

constexpr int SBM = kTcBM;  // 128 rows per tile
constexpr int SBN = kTcBN;  // 64 columns per tile
constexpr int SBK = 16;     // k step through shared memory
constexpr int ST = 256;

// Rows ty + 16 i of warp w are valid for i < imax: a warp holds ty = 2w, 2w + 1.
__device__ __forceinline__ int warp_imax(int m_valid, int warp) {
    return max(0, min(SBM / 16, (m_valid - 2 * warp + 15) / 16));
}

__global__ void __launch_bounds__(ST, 2) stack_gemm1_f64_kernel(const TcTile* __restrict__ tiles,
                                                                const double* __restrict__ lq,
                                                                const double* __restrict__ x,
                                                                const int64_t* __restrict__ xsrc,
                                                                const int32_t* __restrict__ xstride,
                                                                const int64_t* __restrict__ colbase,
                                                                const int32_t* __restrict__ colstride,
                                                                double* __restrict__ t1) {
    __shared__ double As[SBK][SBM + 1];
    __shared__ double Bs[SBK][SBN + 1];
    const TcTile t = tiles[blockIdx.x];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4, warp = tid >> 5;
    const int ln = tid & 63;  // the B column this thread loads
    const bool nv = ln < t.n_valid;
    const int64_t src = nv ? xsrc[t.out_off + ln] : 0;
    const int32_t str = nv ? xstride[t.out_off + ln] : 0;
    const int imax = warp_imax(t.m_valid, warp);
    double acc[SBM / 16][SBN / 16];
#pragma unroll
    for (int i = 0; i < SBM / 16; ++i)
#pragma unroll
        for (int j = 0; j < SBN / 16; ++j) acc[i][j] = 0.0;
    for (int k0 = 0; k0 < t.k_valid; k0 += SBK) {
        const int kl = min(SBK, t.k_valid - k0);
#pragma unroll
        for (int r = 0; r < SBM * SBK / ST; ++r) {
            const int e = tid + ST * r, k = e & 15, m = e >> 4, kk = k0 + k;
            double v = 0.0;
            if (m < t.m_valid && k < kl)
                v = lq[(((int64_t)t.a_row + (int64_t)(kk >> 6) * t.a_cs + m) << 6) + (kk & 63)];
            As[k][m] = v;
        }
#pragma unroll
        for (int r = 0; r < SBN * SBK / ST; ++r) {
            const int k = (tid >> 6) + 4 * r, kk = k0 + k;
            Bs[k][ln] = (nv && k < kl) ? x[src + (int64_t)kk * str] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SBK; ++k) {
            if (k < kl) {
                double b[SBN / 16];
#pragma unroll
                for (int j = 0; j < SBN / 16; ++j) b[j] = Bs[k][tx + 16 * j];
#pragma unroll
                for (int i = 0; i < SBM / 16; ++i)
                    if (i < imax) {
                        const double a = As[k][ty + 16 * i];
#pragma unroll
                        for (int j = 0; j < SBN / 16; ++j) acc[i][j] = fma(a, b[j], acc[i][j]);
                    }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < SBM / 16; ++i) {
        const int m = ty + 16 * i;
        if (i >= imax || m >= t.m_valid) continue;
#pragma unroll
        for (int j = 0; j < SBN / 16; ++j) {
            const int n = tx + 16 * j;
            if (n < t.n_valid) t1[colbase[t.out_off + n] + (int64_t)(t.ldc + m) * colstride[t.out_off + n]] = acc[i][j];
        }
    }
}

__global__ void __launch_bounds__(ST, 2) stack_gemm3_f64_kernel(const TcTile* __restrict__ tiles,
                                                                const double* __restrict__ t2,
                                                                const double* __restrict__ rq,
                                                                const int64_t* __restrict__ yrow,
                                                                double* __restrict__ y) {
    __shared__ double As[SBK][SBM + 1];
    __shared__ double Bs[SBK][SBN + 1];
    const TcTile t = tiles[blockIdx.x];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4, warp = tid >> 5;
    const int imax = warp_imax(t.m_valid, warp);
    double acc[SBM / 16][SBN / 16];
#pragma unroll
    for (int i = 0; i < SBM / 16; ++i)
#pragma unroll
        for (int j = 0; j < SBN / 16; ++j) acc[i][j] = 0.0;
    for (int k0 = 0; k0 < t.k_valid; k0 += SBK) {
        const int kl = min(SBK, t.k_valid - k0);
#pragma unroll
        for (int r = 0; r < SBM * SBK / ST; ++r) {
            const int e = tid + ST * r, k = e & 15, m = e >> 4, kk = k0 + k;
            double v = 0.0;
            if (m < t.m_valid && k < kl)
                v = t2[(((int64_t)t.a_row + (int64_t)(kk >> 6) * t.a_cs + m) << 6) + (kk & 63)];
            As[k][m] = v;
        }
#pragma unroll
        for (int r = 0; r < SBN * SBK / ST; ++r) {
            const int e = tid + ST * r, k = e & 15, n = e >> 4, kk = k0 + k;
            double v = 0.0;
            if (n < t.n_valid && k < kl)
                v = rq[(((int64_t)t.b_row + (int64_t)(kk >> 6) * t.b_cs + n) << 6) + (kk & 63)];
            Bs[k][n] = v;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SBK; ++k) {
            if (k < kl) {
                double b[SBN / 16];
#pragma unroll
                for (int j = 0; j < SBN / 16; ++j) b[j] = Bs[k][tx + 16 * j];
#pragma unroll
                for (int i = 0; i < SBM / 16; ++i)
                    if (i < imax) {
                        const double a = As[k][ty + 16 * i];
#pragma unroll
                        for (int j = 0; j < SBN / 16; ++j) acc[i][j] = fma(a, b[j], acc[i][j]);
                    }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < SBM / 16; ++i) {
        const int m = ty + 16 * i;
        if (i >= imax || m >= t.m_valid) continue;
        double* o = y + yrow[t.out_off + m] + t.n0;
#pragma unroll
        for (int j = 0; j < SBN / 16; ++j) {
            const int n = tx + 16 * j;
            if (n < t.n_valid) o[n] = acc[i][j];
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

}  // namespace

struct F64Stack {
    DevBuf<double> lq, rq, t1, t2, coef;
    DevBuf<TcTile> tiles1, tiles3;
    DevBuf<TcCombJob> jobs;
    DevBuf<TcCombTerm> terms;
    DevBuf<int64_t> yrow, colbase, xsrc;
    DevBuf<int32_t> colstride, xstride;
    int n1 = 0, n3 = 0, njobs = 0;
    double bytes[3] = {0.0, 0.0, 0.0};  // per stage, without the psi / y vectors
};

void F64StackDeleter::operator()(F64Stack* p) const { delete p; }

tk_status f64stack_create(const TcTables& C, std::unique_ptr<F64Stack, F64StackDeleter>& out, std::string& err) {
    std::unique_ptr<F64Stack, F64StackDeleter> p(new F64Stack);
    cudaError_t e = cudaSuccess;
    if ((e = p->lq.upload(C.lq64)) != cudaSuccess || (e = p->rq.upload(C.rq64)) != cudaSuccess ||
        (e = p->tiles1.upload(C.tiles1)) != cudaSuccess || (e = p->tiles3.upload(C.tiles3)) != cudaSuccess ||
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
    if (!C.tiles1x.empty() || !C.tiles3f.empty()) {
        err = "stacked FP64 tables with split-copy or fused tiles";
        return TK_ERR_INVALID_ARG;
    }
    // Bytes each stage must move at least: every valid stack element once
    // (a row tile read by several column tiles counts once), T1 written /
    // read once, T2 written / read once.
    auto stack_elems = [](const std::vector<TcTile>& tiles, bool a_side) {
        std::set<int32_t> seen;
        double n = 0.0;
        for (const TcTile& t : tiles)
            if (seen.insert(a_side ? t.a_row : t.b_row).second)
                n += (double)(a_side ? t.m_valid : t.n_valid) * t.k_valid;
        return n;
    };
    double comb_reads = 0.0;
    for (const TcCombJob& j : C.jobs) comb_reads += (double)j.rows * j.cols * (j.term_end - j.term_begin);
    const double t2_elems = stack_elems(C.tiles3, true);
    p->bytes[0] = 8.0 * (stack_elems(C.tiles1, true) + (double)C.t1_total);
    p->bytes[1] = 8.0 * (std::min<double>((double)C.t1_total, comb_reads) + t2_elems);
    p->bytes[2] = 8.0 * (t2_elems + stack_elems(C.tiles3, false));
    p->n1 = (int)C.tiles1.size();
    p->n3 = (int)C.tiles3.size();
    p->njobs = (int)C.jobs.size();
    out = std::move(p);
    return TK_OK;
}

cudaError_t f64stack_stage(F64Stack& p, const double* x, double* y, cudaStream_t s, int stage) {
    if (stage == 0 && p.n1 > 0)
        stack_gemm1_f64_kernel<<<p.n1, ST, 0, s>>>(p.tiles1.p, p.lq.p, x, p.xsrc.p, p.xstride.p, p.colbase.p,
                                                   p.colstride.p, p.t1.p);
    else if (stage == 1 && p.njobs > 0)
        stack_combine_f64_kernel<<<p.njobs, 128, 0, s>>>(p.jobs.p, p.terms.p, p.coef.p, p.t1.p, p.t2.p);
    else if (stage == 2 && p.n3 > 0)
        stack_gemm3_f64_kernel<<<p.n3, ST, 0, s>>>(p.tiles3.p, p.t2.p, p.rq.p, p.yrow.p, y);
    return cudaGetLastError();
}

cudaError_t f64stack_apply(F64Stack& p, const double* x, double* y, cudaStream_t s) {
    for (int stage = 0; stage < 3; ++stage) {
        cudaError_t e = f64stack_stage(p, x, y, s, stage);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

int f64stack_launches(const F64Stack& p) { return (p.n1 > 0) + (p.njobs > 0) + (p.n3 > 0); }

void f64stack_bytes(const F64Stack& p, double out[3]) {
    for (int i = 0; i < 3; ++i) out[i] = p.bytes[i];
}

}  // namespace tk
