// noalloc.cu -- tk_gemm_f64_noalloc: the FP64 GEMM of tk_gemm_f64 without any
// memory allocation.
//
// Who needs it: callers that must not allocate device memory at call time.
// A sweep that works out of a pre-sized arena (tensorkraft's SweepArena
// design forbids allocation inside the Krylov loop), a host runtime that
// hands the library only the memory it manages itself, and latency-bound
// loops where a cudaMalloc/cudaFree pair per call (what tk_gemm_f64 does for
// its tile tables) costs more than the GEMM.
//
// How: the tile tables the grouped GEMM kernel reads live in one file-scope
// device array, g_noalloc_gemm_scratch, of kNoallocScratchBytes (1 MiB), which
// every GPU that loads this library holds until the process exits.  A small
// kernel writes the task, segment and tile entries into it from kernel
// arguments, then the same grouped GEMM kernel as tk_gemm_f64 runs on the
// caller's stream.  Nothing is allocated, freed or copied from the host.
//
// Limits and rules:
//   * at most kNoallocMaxTiles 64x64 output tiles per call (an output of up
//     to about 16k x 16k); larger calls are rejected with TK_ERR_INVALID_ARG;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current) -- make that first call
//     before any stream capture;
//   * all calls on a device share the one array, which keeps the last call's
//     tables: calls whose work overlaps on the GPU (different streams without
//     ordering between them) race on it; calls on one stream are ordered;
//   * the call is stream-ordered and does not synchronise: C is complete when
//     the stream reaches the end of the call's work;
//   * the array's address is cached per device for the life of the process:
//     after cudaDeviceReset (or any reset of the device's primary context) the
//     module is loaded again at another address, and this entry point must not
//     be called again in that process.
#include <cuda_runtime.h>

#include <climits>
#include <cstdlib>
#include <mutex>
#include <string>

#include "kernels.cuh"
#include "tk_internal.hpp"

namespace {

constexpr size_t kNoallocScratchBytes = 1u << 20;
constexpr size_t kNoallocHeader = 256;  // one GemmTask and one GemmSeg, 256-byte aligned
constexpr int64_t kNoallocMaxTiles = (int64_t)((kNoallocScratchBytes - kNoallocHeader) / sizeof(tk::GemmTile));
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_gemm_scratch[kNoallocScratchBytes];

std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Writes the GEMM's task, its single K segment and the tile list into the scratch.
__global__ void fill_gemm_tables_kernel(tk::GemmTask task, tk::GemmSeg seg, int ntile_n, int ntiles,
                                        unsigned char* scratch) {
    tk::GemmTask* t = reinterpret_cast<tk::GemmTask*>(scratch);
    tk::GemmSeg* s = reinterpret_cast<tk::GemmSeg*>(scratch + 128);
    tk::GemmTile* tiles = reinterpret_cast<tk::GemmTile*>(scratch + kNoallocHeader);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *t = task;
        *s = seg;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ntiles; i += gridDim.x * blockDim.x)
        tiles[i] = tk::GemmTile{0, (i / ntile_n) * tk::kF64TileM, (i % ntile_n) * tk::kF64TileN, 0};
}

tk_status fail(const std::string& msg, tk_status code) {
    tk::set_error(msg);
    return code;
}

}  // namespace

extern "C" tk_status tk_gemm_f64_noalloc(tk_ctx* ctx, double alpha, const tk_mat* a, const tk_mat* b, double beta,
                                         tk_mat_mut* c, void* stream) {
    if (!a || !b || !c || !a->data || !b->data || !c->data)
        return fail("tk_gemm_f64_noalloc: null argument", TK_ERR_INVALID_ARG);
    if (a->cols != b->rows || c->rows != a->rows || c->cols != b->cols)
        return fail("tk_gemm_f64_noalloc: shape mismatch", TK_ERR_INVALID_ARG);
    if (c->rows == 0 || c->cols == 0) return TK_OK;
    const int64_t lim = INT32_MAX;
    if (a->rows > lim || a->cols > lim || b->cols > lim || std::llabs(a->row_stride) > lim ||
        std::llabs(a->col_stride) > lim || std::llabs(b->row_stride) > lim || std::llabs(b->col_stride) > lim ||
        std::llabs(c->row_stride) > lim || std::llabs(c->col_stride) > lim)
        return fail("tk_gemm_f64_noalloc: dimensions or strides exceed 32 bits", TK_ERR_UNSUPPORTED);
    const int64_t ntm = (c->rows + tk::kF64TileM - 1) / tk::kF64TileM;
    const int64_t ntn = (c->cols + tk::kF64TileN - 1) / tk::kF64TileN;
    if (ntm * ntn > kNoallocMaxTiles)
        return fail("tk_gemm_f64_noalloc: output needs " + std::to_string(ntm * ntn) + " 64x64 tiles, more than the " +
                        std::to_string(kNoallocMaxTiles) + " the 1 MiB no-allocation scratch holds; use tk_gemm_f64",
                    TK_ERR_INVALID_ARG);
    const int dev = ctx ? ctx->device : 0;
    if (dev < 0 || dev >= kMaxDevices) return fail("tk_gemm_f64_noalloc: device index out of range", TK_ERR_INVALID_ARG);
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) return fail(std::string("tk_gemm_f64_noalloc: cudaSetDevice: ") + cudaGetErrorString(e), TK_ERR_CUDA);
    struct Restore {
        int d;
        ~Restore() {
            if (d >= 0) cudaSetDevice(d);
        }
    } restore{prev};
    unsigned char* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_ptr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_gemm_scratch);
            if (e != cudaSuccess || !p)
                return fail(std::string("tk_gemm_f64_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e),
                            TK_ERR_CUDA);
            g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
        }
        scratch = g_scratch_ptr[dev];
    }
    tk::GemmTask task{};
    task.M = (int32_t)a->rows;
    task.N = (int32_t)b->cols;
    task.c_off = 0;
    task.c_rs = (int32_t)c->row_stride;
    task.c_cs = (int32_t)c->col_stride;
    task.alpha = alpha;
    task.beta = beta;
    task.seg_begin = 0;
    task.seg_end = a->cols > 0 ? 1 : 0;
    tk::GemmSeg seg{};
    seg.a_off = 0;
    seg.a_rs = (int32_t)a->row_stride;
    seg.a_cs = (int32_t)a->col_stride;
    seg.b_off = 0;
    seg.b_rs = (int32_t)b->row_stride;
    seg.b_cs = (int32_t)b->col_stride;
    seg.K = (int32_t)a->cols;
    const int ntiles = (int)(ntm * ntn);
    cudaStream_t s = (cudaStream_t)stream;
    const int fill_blocks = (ntiles + 255) / 256;
    fill_gemm_tables_kernel<<<fill_blocks, 256, 0, s>>>(task, seg, (int)ntn, ntiles, scratch);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return fail(std::string("tk_gemm_f64_noalloc: table fill launch: ") + cudaGetErrorString(e), TK_ERR_CUDA);
    e = tk::launch_gemm_f64(reinterpret_cast<const tk::GemmTile*>(scratch + kNoallocHeader), ntiles,
                            reinterpret_cast<const tk::GemmTask*>(scratch),
                            reinterpret_cast<const tk::GemmSeg*>(scratch + 128), a->data, b->data, c->data, s);
    if (e != cudaSuccess) return fail(std::string("tk_gemm_f64_noalloc: GEMM launch: ") + cudaGetErrorString(e), TK_ERR_CUDA);
    return TK_OK;
}
