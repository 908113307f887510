// gemm_fp64.cu -- FP64 sector-GEMM path of the two-site H_eff.
//
// grouped_gemm_f64: one CTA per output tile (64, 32 or 16 square, chosen per
// task by the host so small sector blocks are not padded).  A tile's task is one
// output block; its K dimension is a list of segments (one per contributing
// sector pair), accumulated in registers, so every output element is written
// exactly once and no atomics are needed.  Operand tiles are staged through
// shared memory with the load mapping chosen per segment so that the
// unit-stride direction of each operand is the one walked by consecutive
// threads (coalesced for K-major and N-major operands alike).
//
// combine_f64: applies the fused two-site MPO W_ij between the two GEMM
// stages, out = sum_t coef_t * in_t over equally shaped slabs.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.cuh"

namespace tk {

namespace {

constexpr int BK = 16;
constexpr int NT = 256;  // 16 x 16 threads

// One E x E output tile (E = 64, 32 or 16): thread (tx, ty) owns the
// (E/16) x (E/16) outputs (ty + 16 i, tx + 16 j); in a 16 x 16 tile the
// threads are laid over the valid mv x nv outputs instead (thread t owns
// (t / nv, t % nv)), so that a sector block of 13 x 13 keeps six warps
// busy and leaves two idle rather than spreading its outputs over all eight.
// Every output sums its segments in order and k ascending inside each, and
// only the k < K of each segment are multiplied, whatever E and the mapping
// are, so neither changes the result.  Warps without a valid output skip the
// multiplications (the FP64 pipe is this GPU's bottleneck for these tiles).
template <int E>
__device__ __forceinline__ void gemm_tile(const GemmTile& tile, const GemmTask& task, const GemmSeg* __restrict__ segs,
                                          const double* __restrict__ A, const double* __restrict__ B,
                                          double* __restrict__ C, double (*As)[65], double (*Bs)[65], double amul,
                                          int accumulate) {
    constexpr int R = E / 16;
    const int tid = threadIdx.x;
    const int mv = min(E, task.M - tile.m0), nv = min(E, task.N - tile.n0);
    int tx = tid & 15, ty = tid >> 4;
    bool mine = true;
    if (E == 16) {
        mine = tid < mv * nv;
        ty = mine ? tid / nv : 0;
        tx = mine ? tid - ty * nv : 0;
    } else {
        mine = ty < mv && tx < nv;
    }
    const bool warp_busy = __any_sync(0xffffffffu, mine);
    double acc[R][R];
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
        for (int j = 0; j < R; ++j) acc[i][j] = 0.0;

    for (int s = task.seg_begin; s < task.seg_end; ++s) {
        const GemmSeg sg = segs[s];
        for (int k0 = 0; k0 < sg.K; k0 += BK) {
            // A tile: E x BK
#pragma unroll
            for (int r = 0; r < (E * BK) / NT; ++r) {
                int e = tid + r * NT;
                int m, k;
                if (sg.a_cs == 1) { k = e % BK; m = e / BK; } else { m = e % E; k = e / E; }
                int gm = tile.m0 + m, gk = k0 + k;
                double v = 0.0;
                if (gm < task.M && gk < sg.K) v = A[sg.a_off + (int64_t)gm * sg.a_rs + (int64_t)gk * sg.a_cs];
                As[k][m] = v;
            }
            // B tile: BK x E
#pragma unroll
            for (int r = 0; r < (BK * E) / NT; ++r) {
                int e = tid + r * NT;
                int k, n;
                if (sg.b_cs == 1) { n = e % E; k = e / E; } else { k = e % BK; n = e / BK; }
                int gn = tile.n0 + n, gk = k0 + k;
                double v = 0.0;
                if (gn < task.N && gk < sg.K) v = B[sg.b_off + (int64_t)gk * sg.b_rs + (int64_t)gn * sg.b_cs];
                Bs[k][n] = v;
            }
            __syncthreads();
            const int kl = min(BK, sg.K - k0);  // k past the segment's K would add zero products
            if (warp_busy) {
#pragma unroll
                for (int k = 0; k < BK; ++k) {
                    if (k < kl) {
                        double a[R], b[R];
#pragma unroll
                        for (int i = 0; i < R; ++i) a[i] = As[k][ty + 16 * i];
#pragma unroll
                        for (int j = 0; j < R; ++j) b[j] = Bs[k][tx + 16 * j];
#pragma unroll
                        for (int i = 0; i < R; ++i)
#pragma unroll
                            for (int j = 0; j < R; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
                    }
                }
            }
            __syncthreads();
        }
    }
    if (!mine) return;
#pragma unroll
    for (int i = 0; i < R; ++i) {
        int gm = tile.m0 + ty + 16 * i;
        if (gm >= task.M) continue;
#pragma unroll
        for (int j = 0; j < R; ++j) {
            int gn = tile.n0 + tx + 16 * j;
            if (gn >= task.N) continue;
            double* c = C + task.c_off + (int64_t)gm * task.c_rs + (int64_t)gn * task.c_cs;
            double v = amul * task.alpha * acc[i][j];
            if (accumulate)
                v += *c;
            else if (task.beta != 0.0)
                v += task.beta * *c;
            *c = v;
        }
    }
}

__global__ void __launch_bounds__(NT) grouped_gemm_f64_kernel(const GemmTile* __restrict__ tiles, int n_tiles,
                                                              const GemmTask* __restrict__ tasks,
                                                              const GemmSeg* __restrict__ segs,
                                                              const double* __restrict__ A,
                                                              const double* __restrict__ B,
                                                              double* __restrict__ C, double amul, int accumulate) {
    __shared__ double As[BK][65];
    __shared__ double Bs[BK][65];
    const int tile_id = blockIdx.x;
    if (tile_id >= n_tiles) return;
    const GemmTile tile = tiles[tile_id];
    const GemmTask task = tasks[tile.task];
    switch (tile.cls) {  // block-uniform
    case 1: gemm_tile<32>(tile, task, segs, A, B, C, As, Bs, amul, accumulate); break;
    case 2: gemm_tile<16>(tile, task, segs, A, B, C, As, Bs, amul, accumulate); break;
    default: gemm_tile<64>(tile, task, segs, A, B, C, As, Bs, amul, accumulate); break;
    }
}

__global__ void __launch_bounds__(256) combine_f64_kernel(const CombJob* __restrict__ jobs,
                                                          const CombTerm* __restrict__ terms,
                                                          const double* __restrict__ in,
                                                          double* __restrict__ out) {
    const CombJob j = jobs[blockIdx.x];
    const int nterm = j.term_end - j.term_begin;
    __shared__ CombTerm st[64];
    const int n = j.rows * j.cols;
    for (int t0 = 0; t0 < max(nterm, 1); t0 += 64) {
        const int tn = min(64, nterm - t0);
        __syncthreads();
        if (threadIdx.x < tn) st[threadIdx.x] = terms[j.term_begin + t0 + threadIdx.x];
        __syncthreads();
        for (int e = threadIdx.x; e < n; e += blockDim.x) {
            const int r = e / j.cols, c = e - r * j.cols;
            double acc = 0.0;
            for (int t = 0; t < tn; ++t) acc = fma(st[t].coef, in[st[t].in_off + (int64_t)r * st[t].in_rs + c], acc);
            double* o = out + j.out_off + (int64_t)r * j.out_rs + c;
            *o = (t0 == 0) ? acc : (*o + acc);
        }
    }
}

__global__ void start_vector_kernel(double* v, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] = (double)((i * 7 + 13) % 97) / 97.0 - 0.5;
}

}  // namespace

cudaError_t launch_gemm_f64(const GemmTile* tiles, int n_tiles, const GemmTask* tasks, const GemmSeg* segs,
                            const double* A, const double* B, double* C, cudaStream_t s, double amul,
                            bool accumulate) {
    if (n_tiles <= 0) return cudaSuccess;
    grouped_gemm_f64_kernel<<<n_tiles, NT, 0, s>>>(tiles, n_tiles, tasks, segs, A, B, C, amul, accumulate ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_gemm_c64(const GemmTile* tiles, int n_tiles, const GemmTask* tasks, const GemmSeg* segs,
                            const double* Ar, const double* Ai, const double* Br, const double* Bi, double* Cr,
                            double* Ci, bool conj_a, cudaStream_t s) {
    // (Ar + i Ai)^(*) (Br + i Bi): re = Ar Br -+ Ai Bi, im = Ar Bi +- Ai Br
    const double si = conj_a ? 1.0 : -1.0;
    cudaError_t e;
    if ((e = launch_gemm_f64(tiles, n_tiles, tasks, segs, Ar, Br, Cr, s, 1.0, false)) != cudaSuccess) return e;
    if ((e = launch_gemm_f64(tiles, n_tiles, tasks, segs, Ai, Bi, Cr, s, si, true)) != cudaSuccess) return e;
    if ((e = launch_gemm_f64(tiles, n_tiles, tasks, segs, Ar, Bi, Ci, s, 1.0, false)) != cudaSuccess) return e;
    return launch_gemm_f64(tiles, n_tiles, tasks, segs, Ai, Br, Ci, s, -si, true);
}

cudaError_t launch_combine_f64(const CombJob* jobs, int n_jobs, const CombTerm* terms, const double* in,
                               double* out, cudaStream_t s) {
    if (n_jobs <= 0) return cudaSuccess;
    combine_f64_kernel<<<n_jobs, 256, 0, s>>>(jobs, terms, in, out);
    return cudaGetLastError();
}

cudaError_t launch_fill_start_vector(double* v, int64_t n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 8);
    start_vector_kernel<<<blocks, 256, 0, s>>>(v, n);
    return cudaGetLastError();
}

}  // namespace tk
