// tk_env.hpp -- host tables of the block-sparse environment operations
// (growth by one site, two-site start vector); see env.cpp.
#pragma once
#include <string>
#include <vector>

#include "tk_internal.hpp"

namespace tk {

// Output tile of the grouped FP64 GEMM kernel these tables feed (64 x 64).
constexpr int kEnvTileM = 64;
constexpr int kEnvTileN = 64;

// Rank-3 MPS site tensor (s, a_L, a_R) with q(s) + q(a_L) = q(a_R): block of
// (physical sector, left sector) -> element offset (row-major (s, a, b)) and
// its right sector.  `data` is a device pointer, never read on the host.
struct Bst3 {
    int kind = 0;
    QIndex legs[3];
    std::vector<int64_t> blk;  // [phys sector * n_left + left sector], -1 if absent
    std::vector<int> right;
    int64_t total = 0;         // end of the last block
    const double* data = nullptr;
};
bool bst3_from_abi(const tk_bst& t, Bst3& o, const char* name, std::string& err);

// One environment growth: T1 = stage-1 GEMM, T2 = channel combine of T1,
// output = stage-3 GEMM of T2, in the canonical block layouts.
struct GrowTables {
    GemmTable g1, g3;
    std::vector<CombJob> jobs;
    std::vector<CombTerm> terms;
    int64_t t1_total = 0, t2_total = 0, in_total = 0, out_total = 0;
    double comb_flops = 0.0;
};
// left = true: L' from L (on A's left bond) ; false: R' from R (on A's right bond).
tk_status build_grow_tables(bool left, const QIndex& env_bra, const QIndex& env_mpo, const QIndex& env_ket,
                            const Bst3& A, const Bst4& W, GrowTables& G, std::string& err);

// psi(s_i, s_j, a, b) = sum_c A_i(s_i, a, c) A_j(s_j, c, b) into a plan's block layout.
tk_status build_product_tables(const Heff2Tables& H, const Bst3& Ai, const Bst3& Aj, GemmTable& g, std::string& err);

}  // namespace tk
