// tc_gemm.cu -- split-precision (bf16x3) sector GEMMs on tcgen05 tensor cores.
//
// Every FP64 operand x is split into bf16 hi = rn(x) and lo = rn(x - hi);
// a product a*b is evaluated as hi_a*hi_b + hi_a*lo_b + lo_a*hi_b with fp32
// accumulation in tensor memory (the lo*lo term, ~2^-16 relative, is dropped).
//
// One matvec = two to six launches on one stream:
//   split_psi_kernel   psi sub-blocks of tall stage-1 stacks -> bf16 hi/lo copy
//   tc_gemm_kernel     stage 1 of the tall stacks, B operand from that copy
//   tc_gemm1_kernel    stage 1, T1 = L_stack(A) * psi_A        (fp32 out); the
//                      psi operand is read from the fp64 vector and split into
//                      bf16 hi/lo in shared memory by the kernel itself
//   combine_tc_kernel  W_i*W_j channel combine, T1 -> stage-3 A operand hi/lo
//                      (stage-3 stacks wider than TcOptions::fuse_max_ntiles column tiles)
//   tc_gemm3f_kernel   stage 3 of the narrow stacks with the combine fused in:
//                      T2 built in shared memory from T1, then y = T2 * R^T
//   tc_gemm_kernel     stage 3 of the wide stacks, y = T2_stack(B') * R_stack(B')^T
//                      (fp64 out via a row table)
// A stage-1 stack of more than TcOptions::tall_max_mtiles row tiles would have every row
// tile split the same psi columns again; those stacks (the large sectors of
// wide bonds) take the split copy, made once per matvec, instead.
//
// tc_gemm_kernel: one CTA (4 warps) per 128 x 64 output tile.  Warp 0 lane 0
// streams 64-wide K chunks of A_hi, A_lo, B_hi, B_lo with TMA (128-byte
// swizzle) into a two-stage shared-memory ring; warp 1 allocates 64 TMEM
// columns and lane 0 issues three tcgen05.mma (kind::f16, bf16 in, fp32
// accumulate, M=128, N=64, K=16) per 16-wide K step; all four warps read the
// accumulator back with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31) and
// store it.  Every mbarrier wait is bounded: on timeout the kernel records an
// error word, drains what it issued (again bounded), frees its TMEM and exits.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>

#include "tc_gemm.cuh"
#include "tk_plan.cuh"

namespace tk {

namespace {

constexpr int A_BYTES = kTcBM * kTcBK * 2;          // 16 KB (one of hi / lo)
constexpr int B_BYTES = kTcBN * kTcBK * 2;          // 8 KB
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
// Shared memory of an NST-stage pipeline (+ alignment slack and barriers).
// One stage (K <= 64, every stage-1 tile of the U(1)xU(1) workloads) fits
// four CTAs per SM; two stages fit two.
constexpr int smem_bytes(int nst) { return nst * STAGE_BYTES + 1024 + 256; }
constexpr int TMEM_COLS = kTcBN;                    // fp32 accumulator 128 lanes x 64 columns
constexpr long WAIT_LIMIT = 1L << 22;               // bounded mbarrier polls

// error word codes
constexpr int ERR_FULL_TIMEOUT = 1, ERR_EMPTY_TIMEOUT = 2, ERR_DONE_TIMEOUT = 3;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait; false (and the error word set) on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code) {
    for (long i = 0; i < WAIT_LIMIT; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    atomicCAS(err, 0, code);
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, rows of
// 128 bytes, 8-row core groups 1024 bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(16u >> 4) << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// The same for K-major rows of 64 bytes (32 bf16) with the 64-byte swizzle:
// 8-row core groups 512 bytes apart, layout type 4.
__device__ __forceinline__ uint64_t sw64_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(16u >> 4) << 16;
    d |= (uint64_t)(512u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)4 << 61;
    return d;
}

// Instruction descriptor, kind::f16: fp32 accumulate, bf16 A and B, both
// K-major, N>>3 at bit 17, M>>4 at bit 24.  N is chosen per tile.
__device__ __forceinline__ uint32_t make_idesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTcBM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accum) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Programmatic dependent launch: the four kernels of a matvec are launched
// with programmatic stream serialisation, so a kernel's prologue (tables,
// barriers, TMEM) overlaps the previous kernel's tail.  Every kernel calls
// grid_dep_wait() before it reads or writes any buffer another kernel of the
// stream touches; the wait returns once the previous grid has completed and
// its memory is visible, which orders the whole stream transitively.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// 16 consecutive accumulator columns of this thread's TMEM lane (no wait).
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

// Accumulator row of this thread (n_mma <= kTcBN columns) -> srow: every
// tcgen05.ld is issued before the one wait.  Warp-collective (n_mma is
// uniform across the warp).
__device__ __forceinline__ void tmem_row_to_smem(uint32_t tbase, int n_mma, float* srow) {
    uint32_t r[kTcBN];
#pragma unroll
    for (int q = 0; q < kTcBN / 16; ++q)
        if (16 * q < n_mma) tmem_ld16_nowait(tbase + 16 * q, r + 16 * q);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < kTcBN / 16; ++q)
        if (16 * q < n_mma)
#pragma unroll
            for (int i = 0; i < 16; ++i) srow[16 * q + i] = __uint_as_float(r[16 * q + i]);
}

// fp64 -> fp32 on the integer pipes.  This GPU's FP64 pipe is narrow (a few
// operations per SM and clock) and the hardware conversion issues to it, so
// the per-element conversions of the psi split are done from the IEEE 754
// bit layouts instead (fp32 -> fp64 in the epilogues, one per output
// element, stays on the hardware conversion).
//
// fp64 -> fp32, round to nearest even (IEEE 754-2008 default rounding): equal
// to __double2float_rn for every finite input whose result is a normal fp32;
// results below the normal fp32 range (|x| < 2^-126) flush to a signed zero,
// results above it become +-inf; inf and NaN map to inf and a quiet NaN.
__device__ __forceinline__ float d2f_bits(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const uint32_t e = (uint32_t)(b >> 52) & 0x7FFu;
    if (e - 897u < 254u) {
        // normal fp32 range: add the round-to-nearest-even bias below the 23
        // kept mantissa bits (a carry runs into the exponent), keep bits
        // 29.. and rebias the exponent (1023 - 127 = 896) modulo 2^32
        const unsigned long long r = b + (0x0FFFFFFFull + ((b >> 29) & 1ull));
        return __uint_as_float((((uint32_t)(r >> 29)) - (896u << 23)) | sign);
    }
    if (e == 0x7FFu) return __uint_as_float(sign | 0x7F800000u | ((b & 0xFFFFFFFFFFFFFull) ? 0x400000u : 0u));
    return __uint_as_float(e > 896u ? (sign | 0x7F800000u) : sign);  // overflow, or zero / below 2^-126
}


// Two elements at once: x ~ hi + lo with hi = bf16(x32), lo = bf16(x32 - hi),
// x32 = fp32(x) (the difference is exact in fp32); the hi and lo of a and b
// are packed in pairs, a in the low half.
__device__ __forceinline__ void split2x2(double a, double b, uint32_t& hi, uint32_t& lo) {
    const float fa = d2f_bits(a), fb = d2f_bits(b);
    const __nv_bfloat162 h = __floats2bfloat162_rn(fa, fb);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(fa - hf.x, fb - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

// Output addressing of a tile element (row, col) relative to the tile origin.
struct OutMap {
    float* out32;
    double* out64;
    const int64_t* rowtab;
    const int64_t* colbase;
    const int32_t* colstride;
};

__device__ __forceinline__ void store_out(const TcTile& t, int row, int col, float v, const OutMap& o) {
    if (t.mode == 2)
        o.out32[o.colbase[t.out_off + col] + (int64_t)(t.ldc + row) * o.colstride[t.out_off + col]] = v;
    else
        o.out64[o.rowtab[t.out_off + row] + t.n0 + col] = (double)v;
}

// Operands a launch may read before its dependency wait: they are plan
// constants (the split L or R operand), not written by any kernel.
constexpr int CONST_A = 1, CONST_B = 2;

template <int NST>
__global__ void __launch_bounds__(128, 1) tc_gemm_kernel(const TcTile* __restrict__ tiles,
                                                         const __grid_constant__ CUtensorMap mAh,
                                                         const __grid_constant__ CUtensorMap mAl,
                                                         const __grid_constant__ CUtensorMap mBh,
                                                         const __grid_constant__ CUtensorMap mBl, const OutMap om,
                                                         int const_ops, int* err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + NST * STAGE_BYTES);
    uint64_t* empty = full + NST;
    uint64_t* done = empty + NST;
    uint32_t* tslot = (uint32_t*)(done + 1);
    const TcTile t = tiles[blockIdx.x];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    grid_dep_launch();

    if (t.kch == 0) {  // no K: the tile is zero
        grid_dep_wait();
        for (int e = threadIdx.x; e < t.m_valid * t.n_valid; e += blockDim.x)
            store_out(t, e / t.n_valid, e % t.n_valid, 0.f, om);
        return;
    }
    // epilogue addressing from the (constant) plan tables, fetched up front:
    // mode 2, lane c (+32) holds output column c's base and stride; mode 1,
    // lane r holds the y offset of accumulator row 32 * warp + r
    int64_t cb[2] = {0, 0};
    int32_t cs[2] = {0, 0};
    int64_t my_row = 0;
    if (t.mode == 2) {
#pragma unroll
        for (int h = 0; h < 2; ++h)
            if (lane + 32 * h < t.n_valid) {
                cb[h] = om.colbase[t.out_off + lane + 32 * h];
                cs[h] = om.colstride[t.out_off + lane + 32 * h];
            }
    } else if (warp * 32 + lane < t.m_valid) {
        my_row = om.rowtab[t.out_off + warp * 32 + lane];
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;
    const int nb16 = t.n_mma >> 4;  // 16-row B boxes per operand and chunk
    const uint32_t chunk_bytes = 2 * A_BYTES + 2 * t.n_mma * kTcBK * 2;
    const int npre = min(NST, t.kch);  // chunks whose ring slot is free from the start
    auto load_a = [&](int c, uint8_t* st, uint64_t* bar) {
        const int ya = t.a_row + c * t.a_cs;
        tma_load_2d(st, &mAh, 0, ya, bar);
        tma_load_2d(st + A_BYTES, &mAl, 0, ya, bar);
    };
    auto load_b = [&](int c, uint8_t* st, uint64_t* bar) {
        const int yb = t.b_row + c * t.b_cs;
        for (int i = 0; i < nb16; ++i) {
            tma_load_2d(st + 2 * A_BYTES + i * 16 * 128, &mBh, 0, yb + 16 * i, bar);
            tma_load_2d(st + 2 * A_BYTES + B_BYTES + i * 16 * 128, &mBl, 0, yb + 16 * i, bar);
        }
    };
    if (warp == 0 && lane == 0) {
        // the constant operand of the first chunks goes out before the
        // dependency wait (it overlaps the previous kernel's tail)
        for (int c = 0; c < npre; ++c) {
            uint8_t* st = smem + c * STAGE_BYTES;
            mbar_expect_tx(&full[c], chunk_bytes);
            if (const_ops & CONST_A) load_a(c, st, &full[c]);
            if (const_ops & CONST_B) load_b(c, st, &full[c]);
        }
    }
    grid_dep_wait();
    bool ok = true;

    if (warp == 0 && lane == 0) {
        // producer: TMA loads of the K chunks (A: one 128-row box; B: n_mma/16 16-row boxes)
        for (int c = 0; c < t.kch && ok; ++c) {
            const int s = c % NST;
            uint8_t* st = smem + s * STAGE_BYTES;
            if (c < npre) {
                if (!(const_ops & CONST_A)) load_a(c, st, &full[s]);
                if (!(const_ops & CONST_B)) load_b(c, st, &full[s]);
                continue;
            }
            ok = mbar_wait(&empty[s], ((c / NST) - 1) & 1, err, ERR_EMPTY_TIMEOUT);
            if (!ok) break;
            mbar_expect_tx(&full[s], chunk_bytes);
            load_a(c, st, &full[s]);
            load_b(c, st, &full[s]);
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer: three bf16 products per 16-wide K step
        const uint32_t idesc = make_idesc(t.n_mma);
        for (int c = 0; c < t.kch && ok; ++c) {
            const int s = c % NST;
            ok = mbar_wait(&full[s], (c / NST) & 1, err, ERR_FULL_TIMEOUT);
            if (!ok) break;
            fence_after();
            const uint32_t sa = smem_u32(smem + s * STAGE_BYTES);
            const uint64_t ah = sw128_desc(sa), al = sw128_desc(sa + A_BYTES);
            const uint64_t bh = sw128_desc(sa + 2 * A_BYTES), bl = sw128_desc(sa + 2 * A_BYTES + B_BYTES);
#pragma unroll
            for (int kk = 0; kk < kTcBK / 16; ++kk) {
                const uint64_t adv = (uint64_t)((kk * 32) >> 4);  // 16 bf16 = 32 bytes along K
                mma_bf16(tmem, ah + adv, bh + adv, idesc, (c | kk) != 0);
                mma_bf16(tmem, ah + adv, bl + adv, idesc, 1u);
                mma_bf16(tmem, al + adv, bh + adv, idesc, 1u);
            }
            mma_commit(&empty[s]);
        }
        mma_commit(done);
    }
    __syncwarp();
    // epilogue: thread r owns accumulator row r (TMEM lane r)
    const bool have = mbar_wait(done, 0, err, ERR_DONE_TIMEOUT);
    fence_after();
    // tcgen05.ld is warp-collective: decide per warp
    const bool go = __all_sync(0xffffffffu, have);
    if (go) {
        // Accumulator -> shared memory (the operand ring is free once `done`
        // completed) -> coalesced row stores: thread r of warp w holds row
        // 32w + r after tcgen05.ld; the warp then writes its 32 rows one at a
        // time with consecutive lanes on consecutive columns.
        float (*stile)[kTcBN + 1] = reinterpret_cast<float (*)[kTcBN + 1]>(smem);
        const int row = threadIdx.x;
        const uint32_t tbase = tmem + ((uint32_t)(warp * 32) << 16);
        tmem_row_to_smem(tbase, t.n_mma, stile[row]);
        __syncwarp();
        if (t.mode == 2) {
            const int rend = min(t.m_valid, warp * 32 + 32);
            for (int r = warp * 32; r < rend; ++r)
#pragma unroll
                for (int h = 0; h < 2; ++h)
                    if (lane + 32 * h < t.n_valid)
                        om.out32[cb[h] + (int64_t)(t.ldc + r) * cs[h]] = stile[r][lane + 32 * h];
        } else {
            // y rows unrolled eight at a time (independent shuffle / shared-
            // memory / store chains in flight); fp32 -> fp64 is exact, on the
            // hardware conversion (the FP64 pipe is idle in this epilogue)
#pragma unroll 8
            for (int i = 0; i < 32; ++i) {
                const int r = warp * 32 + i;
                const int64_t rbase = __shfl_sync(0xffffffffu, my_row, i);  // every lane, every row
                if (r < t.m_valid) {
                    double* o = om.out64 + rbase + t.n0;
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                        if (lane + 32 * h < t.n_valid) o[lane + 32 * h] = (double)stile[r][lane + 32 * h];
                }
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 1) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}


// Stage 1 with the psi operand built in shared memory.  The L stack (A) comes
// in by TMA as in tc_gemm_kernel; the B tile (n_mma columns x KW K) is read
// from the fp64 vector by all 128 threads (column n of the tile is
// psi[xsrc[n] + k * xstride[n]], zero past the stack's K), split into bf16
// hi / lo and written in the layout a swizzled TMA load would give: KW = 64,
// row n at n * 128 bytes, its 16-byte chunk j at position j ^ (n % 8)
// (128-byte swizzle); KW = 32, row n at n * 64 bytes, chunk j at
// j ^ ((n / 2) % 4) (64-byte swizzle).  A proxy fence and a block barrier
// hand the tile to the MMA thread.  Loop trip counts stay block-uniform
// (bounded waits are combined with __syncthreads_and) so no thread can be
// left at a barrier.
//
// KW = 32 (TcOptions::stage1_narrow) takes the K of a stack in 32-wide
// chunks: chunk c is the half c % 2 of the plan's 64-wide chunk c / 2 (TMA
// box 32 x 128 rows at x = 32 * (c % 2)), so a stage holds 24 KB instead of
// 48, and with one stage, at most 64 registers a thread and 64 TMEM columns a
// CTA, eight CTAs share an SM instead of four.  The MMAs are the same ones in
// the same order, so T1 is bit-identical to KW = 64.
template <int KW>
constexpr int s1_stage_bytes() { return 2 * kTcBM * KW * 2 + 2 * kTcBN * KW * 2; }
template <int KW>
constexpr int s1_smem_bytes(int nst) { return nst * s1_stage_bytes<KW>() + 1024 + 256; }

template <int NST, int KW>
__global__ void __launch_bounds__(128, KW == 64 ? 4 : 8) tc_gemm1_kernel(const TcTile* __restrict__ tiles,
                                                          const __grid_constant__ CUtensorMap mAh,
                                                          const __grid_constant__ CUtensorMap mAl,
                                                          const double* __restrict__ x,
                                                          const int64_t* __restrict__ xsrc,
                                                          const int32_t* __restrict__ xstride, const OutMap om,
                                                          int* err) {
    static_assert(KW == 64 || KW == 32, "stage-1 K chunk of 64 or 32");
    constexpr int A_B = kTcBM * KW * 2, B_B = kTcBN * KW * 2, SB = s1_stage_bytes<KW>();
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + NST * SB);
    uint64_t* empty = full + NST;
    uint64_t* done = empty + NST;
    uint32_t* tslot = (uint32_t*)(done + 1);
    const TcTile t = tiles[blockIdx.x];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    grid_dep_launch();
    // K chunks of this tile (the plan counts 64-wide ones)
    const int kch = KW == 64 ? t.kch : (t.k_valid + KW - 1) / KW;

    if (t.kch == 0) {
        grid_dep_wait();
        for (int e = threadIdx.x; e < t.m_valid * t.n_valid; e += blockDim.x)
            store_out(t, e / t.n_valid, e % t.n_valid, 0.f, om);
        return;
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = make_idesc(t.n_mma);
    // B fill assignment: thread -> one tile column and every fill_step-th k pair
    const int tid = (int)threadIdx.x;
    const int fill_step = 128 / t.n_mma;
    const int fill_col = tid < fill_step * t.n_mma ? tid % t.n_mma : -1;
    const int fill_kq0 = tid / t.n_mma;
    const bool fill_valid = fill_col >= 0 && fill_col < t.n_valid;
    const int64_t fill_src = fill_valid ? xsrc[t.out_off + fill_col] : 0;
    const int64_t fill_stp = fill_valid ? xstride[t.out_off + fill_col] : 0;
    // epilogue: lane c (+32) holds output column c's T1 base and stride
    int64_t cb[2] = {0, 0};
    int32_t cs[2] = {0, 0};
#pragma unroll
    for (int h = 0; h < 2; ++h)
        if (lane + 32 * h < t.n_valid) {
            cb[h] = om.colbase[t.out_off + lane + 32 * h];
            cs[h] = om.colstride[t.out_off + lane + 32 * h];
        }
    // the L operand (a plan constant) of the first chunks goes out before the
    // dependency wait, overlapping the previous kernel's tail
    const int npre = min(NST, kch);
    if (threadIdx.x == 0)
        for (int c = 0; c < npre; ++c) {
            uint8_t* st = smem + c * SB;
            mbar_expect_tx(&full[c], 2 * A_B);
            const int xa = KW == 64 ? 0 : (c & 1) * KW;
            const int ya = t.a_row + (KW == 64 ? c : c >> 1) * t.a_cs;
            tma_load_2d(st, &mAh, xa, ya, &full[c]);
            tma_load_2d(st + A_B, &mAl, xa, ya, &full[c]);
        }
    grid_dep_wait();
    for (int c = 0; c < kch; ++c) {
        const int s = c % NST;
        bool good = true;
        if (c >= NST) good = mbar_wait(&empty[s], ((c / NST) - 1) & 1, err, ERR_EMPTY_TIMEOUT);
        if (!__syncthreads_and(good)) break;
        uint8_t* st = smem + s * SB;
        if (threadIdx.x == 0 && c >= npre) {
            mbar_expect_tx(&full[s], 2 * A_B);
            const int xa = KW == 64 ? 0 : (c & 1) * KW;
            const int ya = t.a_row + (KW == 64 ? c : c >> 1) * t.a_cs;
            tma_load_2d(st, &mAh, xa, ya, &full[s]);
            tma_load_2d(st + A_B, &mAl, xa, ya, &full[s]);
        }
        uint8_t* bh = st + 2 * A_B;
        uint8_t* bl = bh + B_B;
        const int kbase = c * KW;
        // 16-wide K steps that hold data: only those are filled and multiplied
        const int ksteps = min(KW / 16, (t.k_valid - kbase + 15) / 16);
        const int nkp = 8 * ksteps;  // k pairs holding data in this chunk
        if (fill_col >= 0) {
            // a thread owns at most kFillPairs k pairs of a chunk (nkp <= KW / 2,
            // fill_step >= 2): every load of the chunk is in flight at once
            constexpr int kFillPairs = KW / 2 / 2;
            double v[kFillPairs][2];
#pragma unroll
            for (int u = 0; u < kFillPairs; ++u) {
                const int kq = fill_kq0 + u * fill_step;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int k = kbase + 2 * kq + h;
                    v[u][h] = (kq < nkp && fill_valid && k < t.k_valid) ? x[fill_src + (int64_t)k * fill_stp] : 0.0;
                }
            }
#pragma unroll
            for (int u = 0; u < kFillPairs; ++u) {
                const int kq = fill_kq0 + u * fill_step;
                if (kq >= nkp) continue;
                uint32_t hw, lw;
                split2x2(v[u][0], v[u][1], hw, lw);
                const int n = fill_col, k = 2 * kq;
                const uint32_t off =
                    KW == 64 ? (uint32_t)n * 128u + ((uint32_t)((k >> 3) ^ (n & 7)) << 4) + (uint32_t)(k & 7) * 2u
                             : (uint32_t)n * 64u + ((uint32_t)((k >> 3) ^ ((n >> 1) & 3)) << 4) + (uint32_t)(k & 7) * 2u;
                *reinterpret_cast<uint32_t*>(bh + off) = hw;
                *reinterpret_cast<uint32_t*>(bl + off) = lw;
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (warp == 1 && lane == 0) {
            if (mbar_wait(&full[s], (c / NST) & 1, err, ERR_FULL_TIMEOUT)) {
                fence_after();
                const uint32_t sa = smem_u32(st);
                auto desc = [](uint32_t a) { return KW == 64 ? sw128_desc(a) : sw64_desc(a); };
                const uint64_t ah = desc(sa), al = desc(sa + A_B);
                const uint64_t bhd = desc(sa + 2 * A_B), bld = desc(sa + 2 * A_B + B_B);
                for (int q = 0; q < ksteps; ++q) {
                    const uint64_t adv = (uint64_t)((q * 32) >> 4);
                    mma_bf16(tmem, ah + adv, bhd + adv, idesc, (c | q) != 0);
                    mma_bf16(tmem, ah + adv, bld + adv, idesc, 1u);
                    mma_bf16(tmem, al + adv, bhd + adv, idesc, 1u);
                }
            }
            mma_commit(&empty[s]);
        }
    }
    if (warp == 1 && lane == 0) mma_commit(done);
    __syncwarp();
    const bool have = mbar_wait(done, 0, err, ERR_DONE_TIMEOUT);
    fence_after();
    const bool go = __all_sync(0xffffffffu, have);
    if (go && KW == 64) {
        float (*stile)[kTcBN + 1] = reinterpret_cast<float (*)[kTcBN + 1]>(smem);
        const int row = threadIdx.x;
        const uint32_t tbase = tmem + ((uint32_t)(warp * 32) << 16);
        tmem_row_to_smem(tbase, t.n_mma, stile[row]);
        __syncwarp();
        const int rend = min(t.m_valid, warp * 32 + 32);
        for (int r = warp * 32; r < rend; ++r)
#pragma unroll
            for (int h = 0; h < 2; ++h)
                if (lane + 32 * h < t.n_valid) om.out32[cb[h] + (int64_t)(t.ldc + r) * cs[h]] = stile[r][lane + 32 * h];
    } else if (go) {
        // 32 columns at a time through a 128 x 33 transpose buffer (17 KB of
        // the 24 KB stage), 16 TMEM columns per load: 64 registers a thread
        float (*stile)[33] = reinterpret_cast<float (*)[33]>(smem);
        const int row = threadIdx.x;
        const uint32_t tbase = tmem + ((uint32_t)(warp * 32) << 16);
        const int rend = min(t.m_valid, warp * 32 + 32);
        for (int h = 0; h < 2; ++h) {
            if (32 * h >= t.n_mma) break;  // block-uniform
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                if (32 * h + 16 * q >= t.n_mma) break;
                uint32_t r16[16];
                tmem_ld16_nowait(tbase + (uint32_t)(32 * h + 16 * q), r16);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int i = 0; i < 16; ++i) stile[row][16 * q + i] = __uint_as_float(r16[i]);
            }
            __syncwarp();
            if (lane + 32 * h < t.n_valid)
                for (int r = warp * 32; r < rend; ++r)
                    om.out32[cb[h] + (int64_t)(t.ldc + r) * cs[h]] = stile[r][lane];
            __syncwarp();
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 1) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// Stage 1 as a persistent, warp-specialised kernel (TcOptions::stage1_persistent).
// Each CTA (two per SM) walks the tiles blockIdx.x, blockIdx.x + gridDim.x, ...
// of the LPT-ordered list with two roles running side by side:
//   warps 4-7 (producers): per 64-wide K chunk, thread 0 of warp 4 issues the
//     TMA of the L operand, all 128 fill the psi operand (as tc_gemm1_kernel
//     does), and lane 0 of warp 5 issues the MMAs into one of two TMEM
//     accumulators (tile i uses accumulator i & 1) and commits the stage and,
//     on a tile's last chunk, the accumulator;
//   warps 0-3 (epilogue): wait for tile i's accumulator, read it into
//     registers, release it, and write T1 through the column tables.
// So the fill and MMAs of tile i + 1 run while tile i's epilogue stores, and
// the TMEM allocation and barrier set-up are paid once per CTA.  Barriers:
// full[s] (TMA bytes of stage s), sfree[s] (the MMAs reading stage s are
// done), afull[b] (accumulator b holds a finished tile), afree[b] (the
// epilogue has read accumulator b; 128 arrivals).  Every wait is bounded: on
// a timeout the error word is set and the role leaves its loop (the
// producers together, through a barrier reduction), the CTA waits (bounded)
// for its own TMA and MMAs in flight, frees its TMEM and returns.
constexpr int kP1Threads = 256;
constexpr int kP1Stile = kTcBM * (kTcBN + 1) * 4;  // epilogue transpose buffer
constexpr int p1_smem_bytes(int nst) { return nst * STAGE_BYTES + kP1Stile + 1024 + 256; }

// AND of `v` over the `count` threads of named barrier `id` (all must arrive).
__device__ __forceinline__ bool named_bar_and(int id, int count, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id), "r"(count)
        : "memory");
    return r != 0;
}

template <int NST>
__global__ void __launch_bounds__(kP1Threads, 2) tc_gemm1p_kernel(const TcTile* __restrict__ tiles, int ntiles,
                                                                  const __grid_constant__ CUtensorMap mAh,
                                                                  const __grid_constant__ CUtensorMap mAl,
                                                                  const double* __restrict__ x,
                                                                  const int64_t* __restrict__ xsrc,
                                                                  const int32_t* __restrict__ xstride,
                                                                  const OutMap om, int* err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float (*stile)[kTcBN + 1] = reinterpret_cast<float (*)[kTcBN + 1]>(smem + NST * STAGE_BYTES);
    uint64_t* full = (uint64_t*)(smem + NST * STAGE_BYTES + kP1Stile);
    uint64_t* sfree = full + NST;
    uint64_t* afull = sfree + NST;
    uint64_t* afree = afull + 2;
    uint64_t* done = afree + 2;
    uint32_t* tslot = (uint32_t*)(done + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    grid_dep_launch();
    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&sfree[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&afull[b], 1);
            mbar_init(&afree[b], 128);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(2 * TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;
    if (warp >= 4) {
        // ---------------------------------------------------------------- producers
        const int ptid = (int)threadIdx.x - 128;
        int g = 0;            // chunks issued by this CTA
        int last_full = -1;   // last chunk whose TMA thread 0 issued (drained at the end)
        bool ok = true;
        bool waited = false;  // the dependency wait (psi is read from the first fill on)
        for (int i = 0, ti = blockIdx.x; ok && ti < ntiles; ++i, ti += gridDim.x) {
            const TcTile t = tiles[ti];
            const int b = i & 1;
            const uint32_t idesc = make_idesc(t.n_mma);
            const int fill_step = 128 / t.n_mma;
            const int fill_col = ptid < fill_step * t.n_mma ? ptid % t.n_mma : -1;
            const int fill_kq0 = ptid / t.n_mma;
            const bool fill_valid = fill_col >= 0 && fill_col < t.n_valid;
            const int64_t fill_src = fill_valid ? xsrc[t.out_off + fill_col] : 0;
            const int64_t fill_stp = fill_valid ? xstride[t.out_off + fill_col] : 0;
            for (int c = 0; c < t.kch; ++c, ++g) {
                const int s = g % NST;
                bool good = true;
                if (g >= NST) good = mbar_wait(&sfree[s], ((g / NST) - 1) & 1, err, ERR_EMPTY_TIMEOUT);
                if (!named_bar_and(1, 128, good)) {
                    ok = false;
                    break;
                }
                uint8_t* st = smem + s * STAGE_BYTES;
                if (ptid == 0) {
                    // the L operand is a plan constant: it may load before the dependency wait
                    mbar_expect_tx(&full[s], 2 * A_BYTES);
                    const int ya = t.a_row + c * t.a_cs;
                    tma_load_2d(st, &mAh, 0, ya, &full[s]);
                    tma_load_2d(st + A_BYTES, &mAl, 0, ya, &full[s]);
                    last_full = g;
                }
                if (!waited) {
                    grid_dep_wait();
                    waited = true;
                }
                uint8_t* bh = st + 2 * A_BYTES;
                uint8_t* bl = bh + B_BYTES;
                const int kbase = c * kTcBK;
                const int ksteps = min(kTcBK / 16, (t.k_valid - kbase + 15) / 16);
                const int nkp = 8 * ksteps;
                if (fill_col >= 0) {
                    constexpr int kFillPairs = kTcBK / 2 / 2;
                    double v[kFillPairs][2];
#pragma unroll
                    for (int u = 0; u < kFillPairs; ++u) {
                        const int kq = fill_kq0 + u * fill_step;
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            const int k = kbase + 2 * kq + h;
                            v[u][h] = (kq < nkp && fill_valid && k < t.k_valid) ? x[fill_src + (int64_t)k * fill_stp]
                                                                               : 0.0;
                        }
                    }
#pragma unroll
                    for (int u = 0; u < kFillPairs; ++u) {
                        const int kq = fill_kq0 + u * fill_step;
                        if (kq >= nkp) continue;
                        uint32_t hw, lw;
                        split2x2(v[u][0], v[u][1], hw, lw);
                        const int n = fill_col, k = 2 * kq;
                        const uint32_t off =
                            (uint32_t)n * 128u + ((uint32_t)((k >> 3) ^ (n & 7)) << 4) + (uint32_t)(k & 7) * 2u;
                        *reinterpret_cast<uint32_t*>(bh + off) = hw;
                        *reinterpret_cast<uint32_t*>(bl + off) = lw;
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                bool mok = true;
                if (ptid == 32) {
                    if (c == 0 && i >= 2) mok = mbar_wait(&afree[b], ((i >> 1) - 1) & 1, err, ERR_EMPTY_TIMEOUT);
                    if (mok) mok = mbar_wait(&full[s], (g / NST) & 1, err, ERR_FULL_TIMEOUT);
                }
                // the fill of every producer is in shared memory before the MMAs read it
                if (!named_bar_and(1, 128, mok)) {
                    ok = false;
                    break;
                }
                if (ptid == 32) {
                    fence_after();
                    const uint32_t sa = smem_u32(st);
                    const uint64_t ah = sw128_desc(sa), al = sw128_desc(sa + A_BYTES);
                    const uint64_t bhd = sw128_desc(sa + 2 * A_BYTES), bld = sw128_desc(sa + 2 * A_BYTES + B_BYTES);
                    const uint32_t acc = tmem + (uint32_t)(b * TMEM_COLS);
                    for (int q = 0; q < ksteps; ++q) {
                        const uint64_t adv = (uint64_t)((q * 32) >> 4);
                        mma_bf16(acc, ah + adv, bhd + adv, idesc, (c | q) != 0);
                        mma_bf16(acc, ah + adv, bld + adv, idesc, 1u);
                        mma_bf16(acc, al + adv, bhd + adv, idesc, 1u);
                    }
                    mma_commit(&sfree[s]);
                    if (c == t.kch - 1) mma_commit(&afull[b]);
                }
            }
        }
        if (!waited) grid_dep_wait();
        // drain: the MMAs this CTA issued, and the TMA of the last chunk per stage
        if (ptid == 32) {
            mma_commit(done);
            mbar_wait(done, 0, err, ERR_DONE_TIMEOUT);
        }
        if (ptid == 0)
            for (int gg = max(0, last_full - NST + 1); gg <= last_full; ++gg)
                mbar_wait(&full[gg % NST], (gg / NST) & 1, err, ERR_FULL_TIMEOUT);
    } else {
        // ---------------------------------------------------------------- epilogue
        grid_dep_wait();  // T1 may still be read by the previous matvec's combine
        const uint32_t lanebase = (uint32_t)(warp * 32) << 16;
        for (int i = 0, ti = blockIdx.x; ti < ntiles; ++i, ti += gridDim.x) {
            const TcTile t = tiles[ti];
            const int b = i & 1;
            int64_t cb[2] = {0, 0};
            int32_t cs[2] = {0, 0};
#pragma unroll
            for (int h = 0; h < 2; ++h)
                if (lane + 32 * h < t.n_valid) {
                    cb[h] = om.colbase[t.out_off + lane + 32 * h];
                    cs[h] = om.colstride[t.out_off + lane + 32 * h];
                }
            const bool have = mbar_wait(&afull[b], (i >> 1) & 1, err, ERR_DONE_TIMEOUT);
            if (!__all_sync(0xffffffffu, have)) break;
            fence_after();
            tmem_row_to_smem(tmem + (uint32_t)(b * TMEM_COLS) + lanebase, t.n_mma, stile[threadIdx.x]);
            fence_before();
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&afree[b])) : "memory");
            __syncwarp();
            const int rend = min(t.m_valid, warp * 32 + 32);
            for (int r = warp * 32; r < rend; ++r)
#pragma unroll
                for (int h = 0; h < 2; ++h)
                    if (lane + 32 * h < t.n_valid)
                        om.out32[cb[h] + (int64_t)(t.ldc + r) * cs[h]] = stile[r][lane + 32 * h];
            __syncwarp();
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TMEM_COLS) : "memory");
    }
}

// Stage 3 with the W_i W_j combine fused in (stacks of at most
// TcOptions::fuse_max_ntiles column tiles).  The R operand (B) comes in by TMA as in
// tc_gemm_kernel; the A operand, T2 = sum_t coef_t * T1, is built chunk by
// chunk in shared memory by all eight warps from the fill segments of the
// tile: the chunk is cleared, every segment element is summed in fp32 from
// T1, split into bf16 hi / lo and stored in the 128-byte-swizzled K-major
// layout a TMA load would give (row m at m * 128 bytes, its 16-byte chunk j
// at position j ^ (m % 8)).  A two-stage ring lets chunk c + 1 be filled
// while the MMAs of chunk c run.  Warps 0-3 read the accumulator back and
// write y through the row table, as tc_gemm_kernel does.  Waits are bounded
// and their trip counts block-uniform.
constexpr int kFusedThreads = 256;
constexpr int kFusedWarps = kFusedThreads / 32;

template <int NST>
__global__ void __launch_bounds__(kFusedThreads, 2) tc_gemm3f_kernel(const TcTile* __restrict__ tiles,
                                                                    const int32_t* __restrict__ fill_chunk,
                                                                    const TcFillSeg* __restrict__ segs,
                                                                    const TcCombTerm* __restrict__ terms,
                                                                    const float* __restrict__ t1,
                                                                    const __grid_constant__ CUtensorMap mBh,
                                                                    const __grid_constant__ CUtensorMap mBl,
                                                                    const OutMap om, int* err) {
    constexpr int U = 4;  // elements per lane in flight
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + NST * STAGE_BYTES);
    uint64_t* empty = full + NST;
    uint64_t* done = empty + NST;
    uint32_t* tslot = (uint32_t*)(done + 1);
    const TcTile t = tiles[blockIdx.x];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    grid_dep_launch();

    if (t.kch == 0) {
        grid_dep_wait();
        for (int e = threadIdx.x; e < t.m_valid * t.n_valid; e += blockDim.x)
            store_out(t, e / t.n_valid, e % t.n_valid, 0.f, om);
        return;
    }
    int64_t my_row = 0;
    if (warp < 4 && warp * 32 + lane < t.m_valid) my_row = om.rowtab[t.out_off + warp * 32 + lane];
    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;
    const int nb16 = t.n_mma >> 4;
    const uint32_t b_bytes = 2 * t.n_mma * kTcBK * 2;
    auto load_b = [&](int c, uint8_t* st, uint64_t* bar) {
        const int yb = t.b_row + c * t.b_cs;
        for (int i = 0; i < nb16; ++i) {
            tma_load_2d(st + 2 * A_BYTES + i * 16 * 128, &mBh, 0, yb + 16 * i, bar);
            tma_load_2d(st + 2 * A_BYTES + B_BYTES + i * 16 * 128, &mBl, 0, yb + 16 * i, bar);
        }
    };
    // the R operand (a plan constant) of the first chunks goes out before the
    // dependency wait, overlapping the previous kernel's tail
    const int npre = min(NST, t.kch);
    if (threadIdx.x == 0)
        for (int c = 0; c < npre; ++c) {
            mbar_expect_tx(&full[c], b_bytes);
            load_b(c, smem + c * STAGE_BYTES, &full[c]);
        }
    grid_dep_wait();
    const uint32_t idesc = make_idesc(t.n_mma);
    for (int c = 0; c < t.kch; ++c) {
        const int s = c % NST;
        uint8_t* st = smem + s * STAGE_BYTES;
        bool good = true;
        if (c >= NST && threadIdx.x == 0) good = mbar_wait(&empty[s], ((c / NST) - 1) & 1, err, ERR_EMPTY_TIMEOUT);
        if (!__syncthreads_and(good)) break;
        if (threadIdx.x == 0 && c >= npre) {
            mbar_expect_tx(&full[s], b_bytes);
            load_b(c, st, &full[s]);
        }
        // clear A hi / lo: positions no segment covers (K padding, slabs without
        // terms, rows past the stack) must read as zero
        {
            uint4* z = reinterpret_cast<uint4*>(st);
#pragma unroll
            for (int i = 0; i < 2 * A_BYTES / 16 / kFusedThreads; ++i)
                z[threadIdx.x + i * kFusedThreads] = make_uint4(0u, 0u, 0u, 0u);
        }
        __syncthreads();
        const int sb = fill_chunk[t.fill0 + c], se = fill_chunk[t.fill0 + c + 1];
        for (int g = sb + warp; g < se; g += kFusedWarps) {
            const TcFillSeg sg = segs[g];
            const int n = sg.rows * sg.cols;
            const int tb = sg.term_begin, nt = sg.term_end - sg.term_begin;
            for (int e0 = 0; e0 < n; e0 += 32 * U) {
                int r[U], k[U];
                bool v[U];
                float acc[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int e = e0 + u * 32 + lane;
                    v[u] = e < n;
                    r[u] = v[u] ? e / sg.cols : 0;
                    k[u] = v[u] ? e - r[u] * sg.cols : 0;
                    acc[u] = 0.f;
                }
                for (int q = 0; q < nt; ++q) {
                    const TcCombTerm tm = terms[tb + q];
                    float x[U];
#pragma unroll
                    for (int u = 0; u < U; ++u)
                        x[u] = v[u] ? __ldg(t1 + tm.in_off + (int64_t)r[u] * tm.in_rs + k[u]) : 0.f;
#pragma unroll
                    for (int u = 0; u < U; ++u) acc[u] = fmaf(tm.coef, x[u], acc[u]);
                }
#pragma unroll
                for (int u = 0; u < U; ++u)
                    if (v[u]) {
                        const int m = sg.r0 + r[u], kk = sg.k0 + k[u];
                        const uint32_t off =
                            (uint32_t)m * 128u + ((uint32_t)((kk >> 3) ^ (m & 7)) << 4) + (uint32_t)(kk & 7) * 2u;
                        const __nv_bfloat16 h = __float2bfloat16_rn(acc[u]);
                        *reinterpret_cast<__nv_bfloat16*>(st + off) = h;
                        *reinterpret_cast<__nv_bfloat16*>(st + A_BYTES + off) =
                            __float2bfloat16_rn(acc[u] - __bfloat162float(h));
                    }
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (warp == 1 && lane == 0) {
            if (mbar_wait(&full[s], (c / NST) & 1, err, ERR_FULL_TIMEOUT)) {
                fence_after();
                const uint32_t sa = smem_u32(st);
                const uint64_t ah = sw128_desc(sa), al = sw128_desc(sa + A_BYTES);
                const uint64_t bh = sw128_desc(sa + 2 * A_BYTES), bl = sw128_desc(sa + 2 * A_BYTES + B_BYTES);
#pragma unroll
                for (int kk = 0; kk < kTcBK / 16; ++kk) {
                    const uint64_t adv = (uint64_t)((kk * 32) >> 4);
                    mma_bf16(tmem, ah + adv, bh + adv, idesc, (c | kk) != 0);
                    mma_bf16(tmem, ah + adv, bl + adv, idesc, 1u);
                    mma_bf16(tmem, al + adv, bh + adv, idesc, 1u);
                }
            }
            mma_commit(&empty[s]);
        }
    }
    if (warp == 1 && lane == 0) mma_commit(done);
    __syncwarp();
    const bool have = mbar_wait(done, 0, err, ERR_DONE_TIMEOUT);
    fence_after();
    const bool go = __all_sync(0xffffffffu, have);
    if (go && warp < 4) {
        float (*stile)[kTcBN + 1] = reinterpret_cast<float (*)[kTcBN + 1]>(smem);
        const int row = threadIdx.x;
        const uint32_t tbase = tmem + ((uint32_t)(warp * 32) << 16);
        tmem_row_to_smem(tbase, t.n_mma, stile[row]);
        __syncwarp();
#pragma unroll 8
        for (int i = 0; i < 32; ++i) {
            const int r = warp * 32 + i;
            const int64_t rbase = __shfl_sync(0xffffffffu, my_row, i);
            if (r < t.m_valid) {
                double* o = om.out64 + rbase + t.n0;
#pragma unroll
                for (int h = 0; h < 2; ++h)
                    if (lane + 32 * h < t.n_valid) o[lane + 32 * h] = (double)stile[r][lane + 32 * h];
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 1) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

constexpr int kSplitThreads = 128;  // split: threads per job

// psi sub-block tile (64 a x 32 b of a row-major D_A x D_B block, a0 at a K
// chunk boundary) -> 32 rows of the split copy (row = column b, 64 bf16 along
// a), hi and lo.  The tile goes through shared memory so that psi is read
// along b (256-byte row segments) and the copy written along a (four threads
// per 128-byte row, 16-byte stores).  a past D_A is written as zero (K
// padding of that column's own row).
__global__ void __launch_bounds__(kSplitThreads) split_psi_kernel(const TcSplitJob* __restrict__ jobs,
                                                                  const double* __restrict__ x,
                                                                  __nv_bfloat16* __restrict__ xh,
                                                                  __nv_bfloat16* __restrict__ xl) {
    __shared__ double buf[kTcBK][33];
    const TcSplitJob j = jobs[blockIdx.x];
    grid_dep_launch();
    const int na = min(kTcBK, j.rows - j.a0), nb = min(32, j.cols - j.b0);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    grid_dep_wait();
    double v[kTcBK / 4];
#pragma unroll
    for (int u = 0; u < kTcBK / 4; ++u) {
        const int a = w + 4 * u;
        v[u] = (a < na && lane < nb) ? x[j.src + (int64_t)(j.a0 + a) * j.cols + j.b0 + lane] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kTcBK / 4; ++u) buf[w + 4 * u][lane] = v[u];
    __syncthreads();
    const int b = threadIdx.x >> 2, ab = (threadIdx.x & 3) * 16;
    if (b < nb) {
        uint32_t hw[8], lw[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) split2x2(buf[ab + 2 * i][b], buf[ab + 2 * i + 1][b], hw[i], lw[i]);
        const int64_t row = (int64_t)j.xrow + (int64_t)(j.a0 / kTcBK) * j.cstride + j.b0 + b;
        uint4* ph = reinterpret_cast<uint4*>(xh + row * kTcBK + ab);
        uint4* pl = reinterpret_cast<uint4*>(xl + row * kTcBK + ab);
        ph[0] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        ph[1] = make_uint4(hw[4], hw[5], hw[6], hw[7]);
        pl[0] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        pl[1] = make_uint4(lw[4], lw[5], lw[6], lw[7]);
    }
}

constexpr int kCombThreads = 128;  // combine: threads per job

// W_i W_j channel combine: T1 (fp32) -> stage-3 A operand, bf16 hi/lo.  One
// CTA per job (rows [r0, r0 + rows) of one output slab, at most
// kTcCombMaxElems elements unless a single row is longer).  A job of at most
// kTcCombInline terms (most of them: a channel pair reached from one or two
// others) reads its terms from its own descriptor; longer term lists are
// staged in shared memory.  Each thread owns U elements, so a thread has
// TU x U independent T1 loads in flight before the first use.  Elements run
// in row-major order, contiguous in T1 and in the operand chunk.  The kernel
// is bound by its instruction issue: a thread walks its elements (tid, tid +
// 128, ...) by one precomputed quotient and remainder of 128 instead of a
// division per element, and (kWide false: T1 below 2^31 elements) forms
// its T1 and operand offsets in 32 bits.
template <bool kWide>
__device__ __forceinline__ int64_t t1_off(int r, int rs, int c) {
    return kWide ? (int64_t)r * rs + c : (int64_t)(r * rs + c);
}

template <bool kWide, int kThreads = kCombThreads, int U = 4>
__global__ void __launch_bounds__(kThreads, kThreads == 128 ? 12 : 16) combine_tc_kernel(
    const TcCombJob* __restrict__ jobs, const TcCombTerm* __restrict__ terms, const float* __restrict__ t1,
    __nv_bfloat16* __restrict__ th, __nv_bfloat16* __restrict__ tl) {
    constexpr int TU = 2, TCH = 64;
    __shared__ TcCombTerm st[TCH];
    const TcCombJob j = jobs[blockIdx.x];
    grid_dep_launch();
    const int n = j.rows * j.cols;
    const int nterm = j.term_end - j.term_begin;
    // the terms are plan constants: a job with at most TCH of them (and more
    // than kTcCombInline) stages them before the dependency wait
    const bool inl = nterm <= kTcCombInline;
    const bool resident = !inl && nterm <= TCH;
    if (resident && (int)threadIdx.x < nterm) st[threadIdx.x] = terms[j.term_begin + threadIdx.x];
    // element threadIdx.x's (row, column) in the job, and one step of kThreads elements
    const int dq = kThreads / j.cols, dr = kThreads - dq * j.cols;
    int rl = (int)threadIdx.x / j.cols, cl = (int)threadIdx.x - rl * j.cols;
    grid_dep_wait();
    if (resident) __syncthreads();
    if (inl) {
        const float* src[kTcCombInline];
#pragma unroll
        for (int q = 0; q < kTcCombInline; ++q) src[q] = t1 + j.inl[q].in_off;
        for (int e0 = 0; e0 < n; e0 += U * kThreads) {
            bool valid[U];
            int r[U], c[U];
            float acc[U], v[kTcCombInline][U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                valid[u] = e0 + u * kThreads + (int)threadIdx.x < n;
                r[u] = j.r0 + rl;
                c[u] = cl;
                acc[u] = 0.f;
                cl += dr;
                rl += dq;
                if (cl >= j.cols) {
                    cl -= j.cols;
                    ++rl;
                }
            }
#pragma unroll
            for (int q = 0; q < kTcCombInline; ++q)
#pragma unroll
                for (int u = 0; u < U; ++u)
                    v[q][u] = (q < nterm && valid[u]) ? __ldg(src[q] + t1_off<kWide>(r[u], j.inl[q].in_rs, c[u])) : 0.f;
#pragma unroll
            for (int q = 0; q < kTcCombInline; ++q)
                if (q < nterm)
#pragma unroll
                    for (int u = 0; u < U; ++u) acc[u] = fmaf(j.inl[q].coef, v[q][u], acc[u]);
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (valid[u]) {
                    const int k = j.k0 + c[u];
                    const int64_t idx = ((int64_t)(j.t2row + (k >> 6) * j.cstride + r[u]) << 6) + (k & 63);
                    const __nv_bfloat16 h = __float2bfloat16_rn(acc[u]);
                    th[idx] = h;
                    tl[idx] = __float2bfloat16_rn(acc[u] - __bfloat162float(h));
                }
        }
        return;
    }
    for (int e0 = 0; e0 < n; e0 += U * kThreads) {  // block-uniform trip count
        bool valid[U];
        int r[U], c[U];
        float acc[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int e = e0 + u * kThreads + threadIdx.x;
            valid[u] = e < n;
            const int rl = valid[u] ? e / j.cols : 0;
            c[u] = valid[u] ? e - rl * j.cols : 0;
            r[u] = j.r0 + rl;  // row inside the slab
            acc[u] = 0.f;
        }
        for (int t0 = 0; t0 < nterm; t0 += TCH) {
            const int tn = min(TCH, nterm - t0);
            if (!resident) {
                __syncthreads();
                if ((int)threadIdx.x < tn) st[threadIdx.x] = terms[j.term_begin + t0 + threadIdx.x];
                __syncthreads();
            }
            int t = 0;
            for (; t + TU <= tn; t += TU) {
                float v[TU][U];
#pragma unroll
                for (int q = 0; q < TU; ++q) {
                    const int64_t off = st[t + q].in_off;
                    const int rs = st[t + q].in_rs;
#pragma unroll
                    for (int u = 0; u < U; ++u)
                        v[q][u] = valid[u] ? __ldg(t1 + off + (int64_t)r[u] * rs + c[u]) : 0.f;
                }
#pragma unroll
                for (int q = 0; q < TU; ++q)
#pragma unroll
                    for (int u = 0; u < U; ++u) acc[u] = fmaf(st[t + q].coef, v[q][u], acc[u]);
            }
            for (; t < tn; ++t) {
                const int64_t off = st[t].in_off;
                const int rs = st[t].in_rs;
#pragma unroll
                for (int u = 0; u < U; ++u)
                    if (valid[u]) acc[u] = fmaf(st[t].coef, __ldg(t1 + off + (int64_t)r[u] * rs + c[u]), acc[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (valid[u]) {
                const int k = j.k0 + c[u];
                const int64_t idx = (((int64_t)j.t2row + (int64_t)(k >> 6) * j.cstride + r[u]) << 6) + (k & 63);
                const __nv_bfloat16 h = __float2bfloat16_rn(acc[u]);
                th[idx] = h;
                tl[idx] = __float2bfloat16_rn(acc[u] - __bfloat162float(h));
            }
    }
}

// The same combine as persistent warps: every warp takes jobs j = w, w + W,
// ... (W warps in the grid) and loads the T1 values of its next job before it
// sums and stores the current one, so each warp keeps a job's loads in flight
// while the previous job retires (one CTA per job pays every job's load
// latency in full, in several waves of small CTAs).  Jobs of at most
// kTcCombInline terms use their inline terms; longer ones read the rest from
// the table.  Each lane owns elements lane + 32 u of the job (u < 16: jobs
// have at most kTcCombMaxElems elements unless one row is longer, and a
// longer row is walked in further passes).
constexpr int kCombWarpU = kTcCombMaxElems / 32;

struct CombPrefetch {
    float v[kTcCombInline][kCombWarpU];
};

__device__ __forceinline__ void comb_warp_load(const TcCombJob& j, const float* __restrict__ t1, int lane, int e0,
                                               CombPrefetch& p) {
    const int n = j.rows * j.cols;
    const int nterm = min(j.term_end - j.term_begin, kTcCombInline);
#pragma unroll
    for (int u = 0; u < kCombWarpU; ++u) {
        const int e = e0 + u * 32 + lane;
        const bool ok = e < n;
        const int rl = ok ? e / j.cols : 0;
        const int c = ok ? e - rl * j.cols : 0;
        const int r = j.r0 + rl;
#pragma unroll
        for (int q = 0; q < kTcCombInline; ++q)
            p.v[q][u] = (ok && q < nterm) ? __ldg(t1 + j.inl[q].in_off + (int64_t)r * j.inl[q].in_rs + c) : 0.f;
    }
}

__device__ __forceinline__ void comb_warp_store(const TcCombJob& j, const TcCombTerm* __restrict__ terms,
                                                const float* __restrict__ t1, int lane, int e0,
                                                const CombPrefetch& p, __nv_bfloat16* __restrict__ th,
                                                __nv_bfloat16* __restrict__ tl) {
    const int n = j.rows * j.cols;
    const int nterm = j.term_end - j.term_begin;
#pragma unroll
    for (int u = 0; u < kCombWarpU; ++u) {
        const int e = e0 + u * 32 + lane;
        if (e >= n) continue;
        const int rl = e / j.cols;
        const int c = e - rl * j.cols;
        const int r = j.r0 + rl;
        float acc = 0.f;
#pragma unroll
        for (int q = 0; q < kTcCombInline; ++q)
            if (q < nterm) acc = fmaf(j.inl[q].coef, p.v[q][u], acc);
        for (int t = kTcCombInline; t < nterm; ++t) {  // terms past the inline ones
            const TcCombTerm tm = terms[j.term_begin + t];
            acc = fmaf(tm.coef, __ldg(t1 + tm.in_off + (int64_t)r * tm.in_rs + c), acc);
        }
        const int k = j.k0 + c;
        const int64_t idx = (((int64_t)j.t2row + (int64_t)(k >> 6) * j.cstride + r) << 6) + (k & 63);
        const __nv_bfloat16 h = __float2bfloat16_rn(acc);
        th[idx] = h;
        tl[idx] = __float2bfloat16_rn(acc - __bfloat162float(h));
    }
}

__global__ void __launch_bounds__(256, 2) combine_tc_warp_kernel(const TcCombJob* __restrict__ jobs, int njobs,
                                                                const TcCombTerm* __restrict__ terms,
                                                                const float* __restrict__ t1,
                                                                __nv_bfloat16* __restrict__ th,
                                                                __nv_bfloat16* __restrict__ tl) {
    grid_dep_launch();
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int W = gridDim.x * (blockDim.x >> 5);
    grid_dep_wait();
    int j = w;
    if (j >= njobs) return;
    TcCombJob cur = jobs[j];
    CombPrefetch pc;
    comb_warp_load(cur, t1, lane, 0, pc);
    while (true) {
        const int jn = j + W;
        TcCombJob nxt{};
        CombPrefetch pn;
        if (jn < njobs) {
            nxt = jobs[jn];
            comb_warp_load(nxt, t1, lane, 0, pn);
        }
        const int n = cur.rows * cur.cols;
        comb_warp_store(cur, terms, t1, lane, 0, pc, th, tl);
        for (int e0 = 32 * kCombWarpU; e0 < n; e0 += 32 * kCombWarpU) {  // one long row past 512 elements
            CombPrefetch px;
            comb_warp_load(cur, t1, lane, e0, px);
            comb_warp_store(cur, terms, t1, lane, e0, px, th, tl);
        }
        if (jn >= njobs) break;
        j = jn;
        cur = nxt;
        pc = pn;
    }
}

// The same combine with one warp per job (TcOptions::combine_warps == 2).
// The one-CTA-per-job form spends about ninety instructions per element (an
// integer division, 64-bit index arithmetic and the job descriptor in every
// thread) and keeps its issue slots three quarters busy.  Here a lane walks
// elements lane, lane + 32, ... of its warp's job (consecutive lanes on
// consecutive columns, so every load and store instruction stays coalesced),
// stepping its (row, column) by one precomputed quotient and remainder of 32
// instead of dividing, and issues the T1 loads of a group of four elements
// before it sums them.  Elements sum their terms in table order with fmaf, as
// the other forms do (bit-identical T2).  Four jobs per CTA.
constexpr int kWjWarps = 4, kWjG = 4;  // jobs per CTA; elements per lane loaded together

__global__ void __launch_bounds__(32 * kWjWarps) combine_tc_wj_kernel(const TcCombJob* __restrict__ jobs, int njobs,
                                                                    const TcCombTerm* __restrict__ terms,
                                                                    const float* __restrict__ t1,
                                                                    __nv_bfloat16* __restrict__ th,
                                                                    __nv_bfloat16* __restrict__ tl) {
    const int lane = threadIdx.x & 31;
    const int ji = blockIdx.x * kWjWarps + (threadIdx.x >> 5);
    grid_dep_launch();
    if (ji >= njobs) return;
    const TcCombJob j = jobs[ji];  // a plan constant: read before the dependency wait
    const int n = j.rows * j.cols;
    const int nterm = j.term_end - j.term_begin;
    const int dq = 32 / j.cols, dr = 32 - dq * j.cols;  // one step of 32 elements in (rows, columns)
    int rl = lane / j.cols, c = lane - rl * j.cols;
    const float* src0 = t1 + j.inl[0].in_off;
    const float* src1 = t1 + j.inl[1].in_off;
    const int rs0 = j.inl[0].in_rs, rs1 = j.inl[1].in_rs;
    grid_dep_wait();
    for (int e0 = 0; e0 < n; e0 += 32 * kWjG) {  // one pass unless one row is longer than the rest
        float v0[kWjG], v1[kWjG];
        const int rl_start = rl, c_start = c;
#pragma unroll
        for (int g = 0; g < kWjG; ++g) {
            const bool ok = e0 + 32 * g + lane < n;
            const int r = j.r0 + rl;
            v0[g] = (ok && nterm > 0) ? __ldg(src0 + (r * rs0 + c)) : 0.f;
            v1[g] = (ok && nterm > 1) ? __ldg(src1 + (r * rs1 + c)) : 0.f;
            c += dr;
            rl += dq;
            if (c >= j.cols) {
                c -= j.cols;
                ++rl;
            }
        }
        int rg = rl_start, cg = c_start;  // the same walk again for the sums and stores
#pragma unroll
        for (int g = 0; g < kWjG; ++g) {
            if (e0 + 32 * g + lane < n) {
                const int r = j.r0 + rg;
                float acc = 0.f;
                if (nterm > 0) acc = fmaf(j.inl[0].coef, v0[g], acc);
                if (nterm > 1) acc = fmaf(j.inl[1].coef, v1[g], acc);
                for (int t = kTcCombInline; t < nterm; ++t) {  // terms past the inline ones
                    const TcCombTerm tm = terms[j.term_begin + t];
                    acc = fmaf(tm.coef, __ldg(t1 + tm.in_off + (int64_t)r * tm.in_rs + cg), acc);
                }
                const int k = j.k0 + cg;
                const int64_t idx = ((int64_t)(j.t2row + (k >> 6) * j.cstride + r) << 6) + (k & 63);
                const __nv_bfloat16 h = __float2bfloat16_rn(acc);
                th[idx] = h;
                tl[idx] = __float2bfloat16_rn(acc - __bfloat162float(h));
            }
            cg += dr;
            rg += dq;
            if (cg >= j.cols) {
                cg -= j.cols;
                ++rg;
            }
        }
    }
}

template <class T>
cudaError_t put(T** dst, const std::vector<T>& v) {
    *dst = nullptr;
    if (v.empty()) return cudaSuccess;
    cudaError_t e = dev_malloc((void**)dst, sizeof(T) * v.size());
    if (e != cudaSuccess) return e;
    return cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point, so the
// library does not link libcuda directly.
PFN_cuTensorMapEncodeTiled_v12000 encode_fn(std::string& err) {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (fn) return fn;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
        err = "cuTensorMapEncodeTiled entry point unavailable";
        return nullptr;
    }
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    return fn;
}

// A 2D map over an operand of 64-element rows; box_k = 64 (128-byte swizzle)
// or 32 (half a row, 64-byte swizzle: the narrow stage-1 chunks).
bool make_map(CUtensorMap* m, void* ptr, int64_t rows, int box_rows, std::string& err, int box_k = kTcBK) {
    std::memset(m, 0, sizeof(*m));
    if (rows <= 0) return true;
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn(err);
    if (!enc) return false;
    cuuint64_t dims[2] = {(cuuint64_t)kTcBK, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)kTcBK * 2};
    cuuint32_t box[2] = {(cuuint32_t)box_k, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, ptr, dims, strides, box, estr,
                                        CU_TENSOR_MAP_INTERLEAVE_NONE,
                                        box_k == kTcBK ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        err = "cuTensorMapEncodeTiled failed with CUresult " + std::to_string((int)r);
        return false;
    }
    return true;
}

}  // namespace

struct TcPlan {
    TcTile* tiles3f = nullptr;          // fused stage-3 tiles
    int32_t* fill_chunk = nullptr;
    TcFillSeg* fill_segs = nullptr;
    TcCombTerm* fill_terms = nullptr;
    int n3f = 0;
    int comb_form = 0;  // TcOptions::combine_warps: 0 CTA per job, 1 warps, 2 warp per job, 3 64-thread CTA per job
    bool p1 = false;                    // stage 1 as the persistent kernel (TcOptions::stage1_persistent)
    bool narrow1 = false;               // stage 1 in 32-wide K chunks (TcOptions::stage1_narrow)
    int p1_ctas = 0;                    // its resident CTAs per SM x SMs
    bool t1_wide = false;               // T1 holds 2^31 elements or more (64-bit combine offsets)
    __nv_bfloat16 *lh = nullptr, *ll = nullptr, *rh = nullptr, *rl = nullptr;
    __nv_bfloat16 *th = nullptr, *tl = nullptr;
    __nv_bfloat16 *xh = nullptr, *xl = nullptr;  // split copy of psi (tall stage-1 stacks)
    float* t1 = nullptr;
    TcTile *tiles1 = nullptr, *tiles1x = nullptr, *tiles3 = nullptr;
    TcSplitJob* split = nullptr;
    TcCombJob* jobs = nullptr;
    TcCombTerm* terms = nullptr;
    int64_t* yrow = nullptr;
    int64_t* t1col_base = nullptr;
    int32_t* t1col_stride = nullptr;
    int64_t* xsrc = nullptr;
    int32_t* xstride = nullptr;
    int* err = nullptr;
    int n1 = 0, n1x = 0, n3 = 0, nsplit = 0, njobs = 0;
    int32_t n1_cut[kTcPsiPieces + 1] = {};  // tiles1[n1_cut[j], n1_cut[j + 1]) read psi below x_cut[j + 1]
    int64_t x_cut[kTcPsiPieces + 1] = {};
    int nst1 = 1, nst1x = 2, nst3 = 2;  // pipeline stages of the GEMM launches
    CUtensorMap mLh, mLl, mTh, mTl, mRh, mRl, mXh, mXl;
    CUtensorMap mLh32, mLl32;  // the L operand in 32-wide K boxes (narrow stage 1)
    ~TcPlan() {
        void* ps[] = {lh,    ll,    rh,   rl,         th,           tl,   xh,      xl,  t1, tiles1, tiles1x,
                      tiles3, split, jobs, terms, yrow, t1col_base, t1col_stride, xsrc, xstride, err,
                      tiles3f, fill_chunk, fill_segs, fill_terms};
        for (void* p : ps)
            if (p) cudaFree(p);
    }
};

void TcPlanDeleter::operator()(TcPlan* p) const { delete p; }

tk_status tc_plan_create(const Heff2Tables& host, const double*, const double*,
                         std::unique_ptr<TcPlan, TcPlanDeleter>& out, std::string& err) {
    const TcTables& C = host.tc;
    std::unique_ptr<TcPlan, TcPlanDeleter> p(new TcPlan);
    cudaError_t e = cudaSuccess;
    auto bf = [](const std::vector<uint16_t>& v) {
        return std::vector<__nv_bfloat16>(reinterpret_cast<const __nv_bfloat16*>(v.data()),
                                          reinterpret_cast<const __nv_bfloat16*>(v.data()) + v.size());
    };
    auto zeros = [&](__nv_bfloat16** d, int64_t rows) -> cudaError_t {
        *d = nullptr;
        if (rows <= 0) return cudaSuccess;
        cudaError_t r = dev_malloc((void**)d, sizeof(__nv_bfloat16) * kTcBK * (size_t)rows);
        if (r != cudaSuccess) return r;
        return cudaMemset(*d, 0, sizeof(__nv_bfloat16) * kTcBK * (size_t)rows);
    };
    if ((e = put(&p->lh, bf(C.lq_hi))) != cudaSuccess || (e = put(&p->ll, bf(C.lq_lo))) != cudaSuccess ||
        (e = put(&p->rh, bf(C.rq_hi))) != cudaSuccess || (e = put(&p->rl, bf(C.rq_lo))) != cudaSuccess ||
        (e = zeros(&p->th, C.t2q_rows)) != cudaSuccess || (e = zeros(&p->tl, C.t2q_rows)) != cudaSuccess ||
        (e = zeros(&p->xh, C.xq_rows)) != cudaSuccess || (e = zeros(&p->xl, C.xq_rows)) != cudaSuccess ||
        (e = put(&p->tiles1, C.tiles1)) != cudaSuccess || (e = put(&p->tiles3, C.tiles3)) != cudaSuccess ||
        (e = put(&p->tiles1x, C.tiles1x)) != cudaSuccess || (e = put(&p->split, C.split)) != cudaSuccess ||
        (e = put(&p->xsrc, C.xsrc)) != cudaSuccess || (e = put(&p->xstride, C.xstride)) != cudaSuccess ||
        (e = put(&p->jobs, C.jobs)) != cudaSuccess ||
        (e = put(&p->terms, C.terms)) != cudaSuccess || (e = put(&p->yrow, C.yrow)) != cudaSuccess ||
        (e = put(&p->t1col_base, C.t1col_base)) != cudaSuccess ||
        (e = put(&p->t1col_stride, C.t1col_stride)) != cudaSuccess || (e = put(&p->tiles3f, C.tiles3f)) != cudaSuccess ||
        (e = put(&p->fill_chunk, C.fill_chunk)) != cudaSuccess || (e = put(&p->fill_segs, C.fill_segs)) != cudaSuccess ||
        (e = put(&p->fill_terms, C.fill_terms)) != cudaSuccess) {
        err = std::string("tensor-core operand upload: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? TK_ERR_OOM : TK_ERR_CUDA;
    }
    if ((e = dev_malloc((void**)&p->t1, sizeof(float) * (size_t)std::max<int64_t>(C.t1_total, 1))) != cudaSuccess ||
        (e = dev_malloc((void**)&p->err, sizeof(int))) != cudaSuccess || (e = cudaMemset(p->err, 0, sizeof(int))) != cudaSuccess) {
        err = std::string("tensor-core workspace: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? TK_ERR_OOM : TK_ERR_CUDA;
    }
    p->n1 = (int)C.tiles1.size();
    std::copy(C.n1_cut, C.n1_cut + kTcPsiPieces + 1, p->n1_cut);
    std::copy(C.x_cut, C.x_cut + kTcPsiPieces + 1, p->x_cut);
    p->n1x = (int)C.tiles1x.size();
    p->n3 = (int)C.tiles3.size();
    p->n3f = (int)C.tiles3f.size();
    p->t1_wide = C.t1_total > INT32_MAX;
    p->nsplit = (int)C.split.size();
    p->njobs = (int)C.jobs.size();
    p->nst1 = C.max_kch1 <= 1 ? 1 : 2;
    p->nst1x = C.max_kch1x <= 1 ? 1 : 2;
    p->nst3 = C.max_kch3 <= 1 ? 1 : 2;
    if (!make_map(&p->mLh, p->lh, C.lq_rows, kTcBM, err) || !make_map(&p->mLl, p->ll, C.lq_rows, kTcBM, err) ||
        !make_map(&p->mXh, p->xh, C.xq_rows, 16, err) || !make_map(&p->mXl, p->xl, C.xq_rows, 16, err) ||
        !make_map(&p->mTh, p->th, C.t2q_rows, kTcBM, err) || !make_map(&p->mTl, p->tl, C.t2q_rows, kTcBM, err) ||
        !make_map(&p->mRh, p->rh, C.rq_rows, 16, err) || !make_map(&p->mRl, p->rl, C.rq_rows, 16, err) ||
        !make_map(&p->mLh32, p->lh, C.lq_rows, kTcBM, err, 32) || !make_map(&p->mLl32, p->ll, C.lq_rows, kTcBM, err, 32))
        return TK_ERR_CUDA;
    if ((e = cudaFuncSetAttribute(tc_gemm_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(1))) !=
            cudaSuccess ||
        (e = cudaFuncSetAttribute(tc_gemm_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(2))) !=
            cudaSuccess ||
        (e = cudaFuncSetAttribute(tc_gemm1_kernel<1, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  s1_smem_bytes<64>(1))) != cudaSuccess ||
        (e = cudaFuncSetAttribute(tc_gemm1_kernel<2, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  s1_smem_bytes<64>(2))) != cudaSuccess ||
        (e = cudaFuncSetAttribute(tc_gemm1_kernel<1, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  s1_smem_bytes<32>(1))) != cudaSuccess ||
        (e = cudaFuncSetAttribute(tc_gemm3f_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(2))) !=
            cudaSuccess ||
        (e = cudaFuncSetAttribute(tc_gemm1p_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  p1_smem_bytes(1))) != cudaSuccess ||
        (e = cudaFuncSetAttribute(tc_gemm1p_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  p1_smem_bytes(2))) != cudaSuccess) {
        err = std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e);
        return TK_ERR_CUDA;
    }
    tk_status st = tc_set_launch_forms(*p, host.tcopt, err);
    if (st != TK_OK) return st;
    out = std::move(p);
    return TK_OK;
}

tk_status tc_set_launch_forms(TcPlan& p, const TcOptions& o, std::string& err) {
    p.comb_form = o.combine_warps;
    if (p.comb_form == 2 && p.t1_wide) p.comb_form = 0;  // form 2 indexes T1 rows in 32 bits
    p.p1 = o.stage1_persistent != 0;
    p.narrow1 = !p.p1 && o.stage1_narrow != 0;
    if (p.p1 && p.p1_ctas == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaError_t e;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
            (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
            (e = p.nst1 == 1 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tc_gemm1p_kernel<1>, kP1Threads,
                                                                             p1_smem_bytes(1))
                             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tc_gemm1p_kernel<2>, kP1Threads,
                                                                             p1_smem_bytes(2))) != cudaSuccess) {
            err = std::string("persistent stage-1 occupancy: ") + cudaGetErrorString(e);
            return TK_ERR_CUDA;
        }
        p.p1_ctas = std::max(1, per_sm) * std::max(1, sms);
    }
    return TK_OK;
}

namespace {

// Launch with programmatic stream serialisation (see grid_dep_wait).
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

void launch_tc_gemm(int nst, int n, const TcTile* tiles, const CUtensorMap& ah, const CUtensorMap& al,
                    const CUtensorMap& bh, const CUtensorMap& bl, const OutMap& om, int const_ops, int* err,
                    cudaStream_t s) {
    if (n <= 0) return;
    if (nst == 1)
        launch_pdl(tc_gemm_kernel<1>, n, 128, smem_bytes(1), s, tiles, ah, al, bh, bl, om, const_ops, err);
    else
        launch_pdl(tc_gemm_kernel<2>, n, 128, smem_bytes(2), s, tiles, ah, al, bh, bl, om, const_ops, err);
}

}  // namespace

namespace {

void launch_stage1_fused(TcPlan& tc, const double* x, int first, int count, cudaStream_t s) {
    if (count <= 0) return;
    const OutMap om{tc.t1, nullptr, nullptr, tc.t1col_base, tc.t1col_stride};
    const TcTile* tiles = tc.tiles1 + first;
    if (tc.p1) {
        const int grid = std::min(count, tc.p1_ctas);
        if (tc.nst1 == 1)
            launch_pdl(tc_gemm1p_kernel<1>, grid, kP1Threads, p1_smem_bytes(1), s, tiles, count, tc.mLh, tc.mLl, x,
                       (const int64_t*)tc.xsrc, (const int32_t*)tc.xstride, om, tc.err);
        else
            launch_pdl(tc_gemm1p_kernel<2>, grid, kP1Threads, p1_smem_bytes(2), s, tiles, count, tc.mLh, tc.mLl, x,
                       (const int64_t*)tc.xsrc, (const int32_t*)tc.xstride, om, tc.err);
        return;
    }
    if (tc.narrow1)  // one 24 KB stage whatever the tiles' K: the chunks of a tile run one after another
        launch_pdl(tc_gemm1_kernel<1, 32>, count, 128, s1_smem_bytes<32>(1), s, tiles, tc.mLh32, tc.mLl32, x,
                   (const int64_t*)tc.xsrc, (const int32_t*)tc.xstride, om, tc.err);
    else if (tc.nst1 == 1)
        launch_pdl(tc_gemm1_kernel<1, 64>, count, 128, s1_smem_bytes<64>(1), s, tiles, tc.mLh, tc.mLl, x,
                   (const int64_t*)tc.xsrc, (const int32_t*)tc.xstride, om, tc.err);
    else
        launch_pdl(tc_gemm1_kernel<2, 64>, count, 128, s1_smem_bytes<64>(2), s, tiles, tc.mLh, tc.mLl, x,
                   (const int64_t*)tc.xsrc, (const int32_t*)tc.xstride, om, tc.err);
}

}  // namespace

bool tc_psi_pieces(const TcPlan& tc, int k, int64_t* x_cut, int32_t* n1_cut) {
    if (k < 2 || k > kTcPsiPieces || kTcPsiPieces % k != 0 || tc.nsplit > 0 || tc.n1x > 0 || tc.n1 <= 0)
        return false;
    const int step = kTcPsiPieces / k;
    for (int j = 0; j <= k; ++j) {
        x_cut[j] = tc.x_cut[j * step];
        n1_cut[j] = tc.n1_cut[j * step];
    }
    return true;
}

cudaError_t tc_stage1_range(TcPlan& tc, const double* x, int first, int count, cudaStream_t s) {
    launch_stage1_fused(tc, x, first, count, s);
    return cudaGetLastError();
}

cudaError_t tc_apply_stage(TcPlan& tc, const Heff2Tables&, const CombJob*, int, const CombTerm*, const double* x,
                           double* y, cudaStream_t s, int stage, std::string& err) {
    if (stage == 0) {
        const OutMap om{tc.t1, nullptr, nullptr, tc.t1col_base, tc.t1col_stride};
        if (tc.nsplit > 0)
            launch_pdl(split_psi_kernel, tc.nsplit, kSplitThreads, 0, s, (const TcSplitJob*)tc.split, x, tc.xh, tc.xl);
        launch_tc_gemm(tc.nst1x, tc.n1x, tc.tiles1x, tc.mLh, tc.mLl, tc.mXh, tc.mXl, om, CONST_A, tc.err, s);
        launch_stage1_fused(tc, x, 0, tc.n1, s);
    } else if (stage == 1) {
        if (tc.njobs > 0 && tc.comb_form == 2)
            launch_pdl(combine_tc_wj_kernel, (tc.njobs + kWjWarps - 1) / kWjWarps, 32 * kWjWarps, 0, s,
                       (const TcCombJob*)tc.jobs, tc.njobs, (const TcCombTerm*)tc.terms, (const float*)tc.t1,
                       tc.th, tc.tl);
        else if (tc.njobs > 0 && tc.comb_form == 1)
            launch_pdl(combine_tc_warp_kernel, std::min(tc.njobs, 152 * 2 * 8) / 8 + 1, 256, 0, s,
                       (const TcCombJob*)tc.jobs, tc.njobs, (const TcCombTerm*)tc.terms, (const float*)tc.t1,
                       tc.th, tc.tl);
        else if (tc.njobs > 0 && tc.comb_form == 3)
            launch_pdl(tc.t1_wide ? combine_tc_kernel<true, 64, 8> : combine_tc_kernel<false, 64, 8>, tc.njobs, 64, 0,
                       s, (const TcCombJob*)tc.jobs, (const TcCombTerm*)tc.terms, (const float*)tc.t1, tc.th, tc.tl);
        else if (tc.njobs > 0)
            launch_pdl(tc.t1_wide ? combine_tc_kernel<true> : combine_tc_kernel<false>, tc.njobs, kCombThreads, 0, s,
                       (const TcCombJob*)tc.jobs, (const TcCombTerm*)tc.terms, (const float*)tc.t1, tc.th, tc.tl);
    } else {
        // fused tiles first: their dependency is stage 1 (T1); the TMA tiles read
        // the combine's T2, complete before either launch starts its main loop
        if (tc.n3f > 0)
            launch_pdl(tc_gemm3f_kernel<2>, tc.n3f, kFusedThreads, smem_bytes(2), s, (const TcTile*)tc.tiles3f,
                       (const int32_t*)tc.fill_chunk, (const TcFillSeg*)tc.fill_segs,
                       (const TcCombTerm*)tc.fill_terms, (const float*)tc.t1, tc.mRh, tc.mRl,
                       OutMap{nullptr, y, tc.yrow, nullptr, nullptr}, tc.err);
        launch_tc_gemm(tc.nst3, tc.n3, tc.tiles3, tc.mTh, tc.mTl, tc.mRh, tc.mRl,
                       OutMap{nullptr, y, tc.yrow, nullptr, nullptr}, CONST_B, tc.err, s);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) err = "tensor-core stage launch";
    return e;
}

cudaError_t tc_apply(TcPlan& tc, const Heff2Tables& host, const CombJob* d_jobs, int n_jobs, const CombTerm* d_terms,
                     const double* x, double* y, cudaStream_t s, std::string& err) {
    for (int stage = 0; stage < 3; ++stage) {
        cudaError_t e = tc_apply_stage(tc, host, d_jobs, n_jobs, d_terms, x, y, s, stage, err);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

namespace {

// Counts inputs where the integer-pipe conversion differs from the hardware
// one: d2f_bits vs __double2float_rn, on inputs with a normal fp32 result.
__global__ void conversion_check_kernel(const double* __restrict__ x, int64_t n, unsigned long long* bad) {
    unsigned long long cnt = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = x[i];
        const float ref = __double2float_rn(v);
        const float got = d2f_bits(v);
        const bool normal = fabsf(ref) >= 1.17549435e-38f && fabsf(ref) <= 3.40282347e38f;
        if (normal && __float_as_uint(ref) != __float_as_uint(got)) ++cnt;
    }
    if (cnt) atomicAdd(bad, cnt);
}

}  // namespace

cudaError_t tc_conversion_check(const double* x, int64_t n, unsigned long long* bad, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    conversion_check_kernel<<<152 * 4, 256, 0, s>>>(x, n, bad);
    return cudaGetLastError();
}

int* tc_error_word(TcPlan& tc) { return tc.err; }

int tc_launches(const TcPlan& tc) {
    return (tc.nsplit > 0) + (tc.n1x > 0) + (tc.n1 > 0) + (tc.njobs > 0) + (tc.n3f > 0) + (tc.n3 > 0);
}

tk_status tc_check_error(TcPlan& tc, cudaStream_t s) {
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, tc.err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail("tensor-core error word", e);
    if (h != 0) {
        cudaMemsetAsync(tc.err, 0, sizeof(int), s);
        cudaStreamSynchronize(s);
        set_error("tensor-core kernel: a bounded wait ran out (code " + std::to_string(h) +
                  "); the affected output tiles were not written");
        return TK_ERR_TIMEOUT;
    }
    return TK_OK;
}

}  // namespace tk
