// contract.cu -- tk_contract_pairwise_f64: one pairwise step of the
// block-sparse contraction executor on the device.
//
// Reference: SparseContractionExecutor::execute_pairwise_sparse and
// reshape_for_gemm (tk-contract/src/sparse.rs:124-265), which permute each
// operand (BlockSparseTensor::permute, tk-symmetry/src/block_sparse.rs:400-431),
// fuse its free and contracted legs into one leg each
// (BlockSparseTensor::fuse_legs, block_sparse.rs:444-611) and hand the two
// rank-2 tensors to SparseLinAlgBackend::block_gemm.
//
// Here the permute and both fusions are one integer pass on the host that
// yields, for every source block, the rectangle it occupies in its fused
// rank-2 block; the device then gathers every source block into place with
// one launch per operand (a general-rank permutation through per-block stride
// tables), and the same grouped FP64 GEMM as block_gemm multiplies the fused
// operands.  Everything goes through the context's scratch: one host-to-device
// copy in, one device-to-host copy out, no allocation once the scratch is
// large enough.
//
// Layout rules kept from the reference (the result must be bit-identical in
// keys, offsets and block layout):
//   * permutation: free legs in ascending leg order, then the contracted legs
//     in ascending leg order (left operand), or contracted then free (right);
//   * a fused leg (more than one leg fused) is Incoming; its sectors are the
//     distinct fused charges in ascending order, a leg's charge entering as
//     itself if Incoming and as its dual if Outgoing, and inside a fused
//     sector the combinations sit in Cartesian order of the sub-legs' sectors
//     (last sub-leg fastest), every combination counted whether or not a
//     block uses it;
//   * a single leg is not fused (its QIndex and direction stay);
//   * a rank-2 operand whose one contracted leg is already in place is used
//     as it is.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "tk_bsgemm.hpp"
#include "tk_internal.hpp"
#include "tk_plan.cuh"

namespace tk {
namespace {

constexpr int kMaxRank = 8;

// One source block's place in its fused rank-2 block: element (i, j) of the
// rectangle (i over the row legs, j over the column legs, each row-major)
// comes from src[src_off + sum idx_l * stride_l].
struct FusePiece {
    int64_t src_off, dst_off;  // dst_off: the rectangle's first element
    int32_t ld, rows, cols, nr, nc, pad;
    int32_t rdim[kMaxRank], rstr[kMaxRank];
    int32_t cdim[kMaxRank], cstr[kMaxRank];
};

__global__ void fuse_gather_kernel(const FusePiece* __restrict__ pieces, const double* __restrict__ src,
                                   double* __restrict__ dst) {
    const FusePiece& p = pieces[blockIdx.y];
    const int64_t n = (int64_t)p.rows * p.cols;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = e / p.cols, j = e - i * p.cols;
        int64_t so = p.src_off;
        for (int l = p.nc - 1; l >= 0; --l) {
            const int64_t q = j / p.cdim[l];
            so += (j - q * p.cdim[l]) * p.cstr[l];
            j = q;
        }
        for (int l = p.nr - 1; l >= 0; --l) {
            const int64_t q = i / p.rdim[l];
            so += (i - q * p.rdim[l]) * p.rstr[l];
            i = q;
        }
        dst[p.dst_off + (e / p.cols) * p.ld + (e % p.cols)] = src[so];
    }
}

// A block-sparse tensor of any rank read from the ABI (host structure).
struct BstN {
    int kind = 0, rank = 0;
    std::vector<QIndex> legs;
    std::vector<int8_t> dirs;
    Qn flux;
    std::vector<std::array<int, kMaxRank>> sec;  // sector index per leg, per block
    std::vector<int64_t> offs;
    const double* data = nullptr;
    int64_t total = 0;
};

bool bstn_from_abi(const tk_bst& t, BstN& o, const char* name, std::string& err) {
    if (t.rank < 1 || t.rank > kMaxRank || !t.legs || !qn_kind_valid(t.qn_kind) ||
        t.rank * qn_bits(t.qn_kind) > 64) {
        err = std::string(name) + ": rank 1 to 8 (and a packed key within 64 bits) with a known kind required";
        return false;
    }
    o.kind = t.qn_kind;
    o.rank = t.rank;
    o.legs.resize(t.rank);
    o.dirs.resize(t.rank);
    for (int l = 0; l < t.rank; ++l) {
        if (!qindex_from_abi(t.qn_kind, t.legs[l], o.legs[l], err)) {
            err = std::string(name) + ": " + err;
            return false;
        }
        o.dirs[l] = t.leg_dirs ? t.leg_dirs[l] : TK_LEG_INCOMING;
    }
    if (t.flux)
        for (int k = 0; k < qn_ncomp(t.qn_kind); ++k) o.flux.c[k] = t.flux[k];
    if (t.n_blocks > 0 && (!t.keys || !t.block_offsets || !t.data)) {
        err = std::string(name) + ": null block arrays";
        return false;
    }
    o.data = t.data;
    for (int64_t b = 0; b < t.n_blocks; ++b) {
        Qn q[kMaxRank];
        key_unpack(t.qn_kind, t.keys[b], t.rank, q);
        std::array<int, kMaxRank> s{};
        int64_t size = 1;
        for (int l = 0; l < t.rank; ++l) {
            s[l] = o.legs[l].find(q[l]);
            if (s[l] < 0) {
                err = std::string(name) + ": block key names a sector missing from its QIndex";
                return false;
            }
            size *= o.legs[l].dim[s[l]];
        }
        if (b > 0 && t.keys[b - 1] >= t.keys[b]) {
            err = std::string(name) + ": keys not strictly ascending";
            return false;
        }
        if (t.block_offsets[b] < 0 || size > INT32_MAX) {
            err = std::string(name) + ": block offset or size out of range";
            return false;
        }
        o.sec.push_back(s);
        o.offs.push_back(t.block_offsets[b]);
        o.total = std::max(o.total, t.block_offsets[b] + size);
    }
    return true;
}

// A fused leg: QIndex, direction, and where each combination of its sub-legs'
// sectors lands (key = the sub-sector indices packed base n_sectors).
struct FusedLeg {
    QIndex q;
    int8_t dir = TK_LEG_INCOMING;
    std::map<std::vector<int>, std::pair<int, int64_t>> at;  // sub-sectors -> (fused sector, offset)
};

void fuse_leg(int kind, const BstN& t, const std::vector<int>& sub, FusedLeg& f) {
    if (sub.size() == 1) {  // a single leg is not fused
        const int l = sub[0];
        f.q = t.legs[l];
        f.dir = t.dirs[l];
        for (int s = 0; s < t.legs[l].n(); ++s) f.at[{s}] = {s, 0};
        return;
    }
    // Cartesian product of the sub-legs' sectors, last sub-leg fastest
    struct Combo {
        std::vector<int> s;
        Qn q;
        int64_t dim;
    };
    std::vector<Combo> combos{{{}, Qn{}, 1}};
    for (int l : sub) {
        std::vector<Combo> next;
        next.reserve(combos.size() * t.legs[l].n());
        for (const Combo& c : combos)
            for (int s = 0; s < t.legs[l].n(); ++s) {
                Combo n = c;
                n.s.push_back(s);
                const Qn eff = t.dirs[l] == TK_LEG_INCOMING ? t.legs[l].q[s] : qn_dual(kind, t.legs[l].q[s]);
                n.q = qn_fuse(kind, c.q, eff);
                n.dim = c.dim * t.legs[l].dim[s];
                next.push_back(std::move(n));
            }
        combos.swap(next);
    }
    // group by fused charge, ascending; offsets in combination order
    std::vector<Qn> charges;
    for (const Combo& c : combos) charges.push_back(c.q);
    std::sort(charges.begin(), charges.end(), qn_less);
    charges.erase(std::unique(charges.begin(), charges.end()), charges.end());
    std::vector<int64_t> fill(charges.size(), 0);
    for (const Combo& c : combos) {
        const int g = (int)(std::lower_bound(charges.begin(), charges.end(), c.q, qn_less) - charges.begin());
        f.at[c.s] = {g, fill[g]};
        fill[g] += c.dim;
    }
    f.q.q = charges;
    f.q.dim = fill;
    f.q.off.resize(charges.size());
    f.q.total = 0;
    for (size_t g = 0; g < charges.size(); ++g) {
        f.q.off[g] = f.q.total;
        f.q.total += fill[g];
    }
    f.dir = TK_LEG_INCOMING;
}

// reshape_for_gemm: the fused rank-2 operand (structure on the host) and the
// gather pieces that build its data from the source blocks.
struct Fused2 {
    Rank2 m;                       // fused rank-2 tensor (data: device, set later)
    std::vector<FusePiece> pieces; // dst_off relative to the fused buffer
};

tk_status reshape_for_gemm(const BstN& t, const std::vector<int>& contracted, bool contracted_trailing, Fused2& out,
                           std::string& err) {
    const int rank = t.rank;
    std::vector<char> is_c(rank, 0);
    for (int l : contracted) {
        if (l < 0 || l >= rank || is_c[l]) {
            err = "contracted leg out of range or repeated";
            return TK_ERR_INVALID_ARG;
        }
        is_c[l] = 1;
    }
    std::vector<int> freel, contl;
    for (int l = 0; l < rank; ++l) (is_c[l] ? contl : freel).push_back(l);
    if (freel.empty() || contl.empty()) {
        err = "each operand needs at least one free and one contracted leg";
        return TK_ERR_UNSUPPORTED;
    }
    const std::vector<int>& rowl = contracted_trailing ? freel : contl;
    const std::vector<int>& coll = contracted_trailing ? contl : freel;
    FusedLeg fr, fc;
    fuse_leg(t.kind, t, rowl, fr);
    fuse_leg(t.kind, t, coll, fc);
    Rank2& m = out.m;
    m.kind = t.kind;
    m.legs[0] = fr.q;
    m.legs[1] = fc.q;
    m.dirs[0] = fr.dir;
    m.dirs[1] = fc.dir;
    m.flux = t.flux;
    // fused block of every source block; fused blocks ascending by packed key
    struct Src {
        int b, r, c;
        int64_t ro, co;
    };
    std::vector<Src> srcs;
    std::map<uint64_t, std::pair<int, int>> fblocks;  // key -> (row sector, col sector)
    for (size_t b = 0; b < t.sec.size(); ++b) {
        std::vector<int> rs, cs;
        for (int l : rowl) rs.push_back(t.sec[b][l]);
        for (int l : coll) cs.push_back(t.sec[b][l]);
        const auto& ra = fr.at.at(rs);
        const auto& ca = fc.at.at(cs);
        Qn q[2] = {fr.q.q[ra.first], fc.q.q[ca.first]};
        fblocks[key_pack(t.kind, q, 2)] = {ra.first, ca.first};
        srcs.push_back({(int)b, ra.first, ca.first, ra.second, ca.second});
    }
    std::map<std::pair<int, int>, int64_t> foff;
    m.total = 0;
    for (const auto& kv : fblocks) {
        m.keys.push_back(kv.first);
        m.offs.push_back(m.total);
        m.rs.push_back(kv.second.first);
        m.cs.push_back(kv.second.second);
        foff[kv.second] = m.total;
        m.total += fr.q.dim[kv.second.first] * fc.q.dim[kv.second.second];
    }
    for (const Src& sr : srcs) {
        FusePiece p{};
        p.src_off = t.offs[sr.b];
        const int64_t ld = fc.q.dim[sr.c];
        if (ld > INT32_MAX) {
            err = "fused block too wide";
            return TK_ERR_UNSUPPORTED;
        }
        p.ld = (int32_t)ld;
        p.dst_off = foff.at({sr.r, sr.c}) + sr.ro * ld + sr.co;
        // source strides of the block (row-major over the original legs)
        int64_t str[kMaxRank];
        int64_t acc = 1;
        for (int l = rank - 1; l >= 0; --l) {
            str[l] = acc;
            acc *= t.legs[l].dim[t.sec[sr.b][l]];
        }
        int64_t rows = 1, cols = 1;
        p.nr = (int32_t)rowl.size();
        p.nc = (int32_t)coll.size();
        for (int i = 0; i < p.nr; ++i) {
            p.rdim[i] = (int32_t)t.legs[rowl[i]].dim[t.sec[sr.b][rowl[i]]];
            p.rstr[i] = (int32_t)str[rowl[i]];
            rows *= p.rdim[i];
        }
        for (int i = 0; i < p.nc; ++i) {
            p.cdim[i] = (int32_t)t.legs[coll[i]].dim[t.sec[sr.b][coll[i]]];
            p.cstr[i] = (int32_t)str[coll[i]];
            cols *= p.cdim[i];
        }
        p.rows = (int32_t)rows;
        p.cols = (int32_t)cols;
        out.pieces.push_back(p);
    }
    return TK_OK;
}

}  // namespace
}  // namespace tk

using namespace tk;

#define CKC(op)                                          \
    do {                                                 \
        cudaError_t e_ = (op);                           \
        if (e_ != cudaSuccess) return cuda_fail(#op, e_); \
    } while (0)

extern "C" tk_status tk_contract_pairwise_f64(tk_ctx* ctx, const tk_bst* a, const int32_t* a_legs, int32_t n_a,
                                              const tk_bst* b, const int32_t* b_legs, int32_t n_b, tk_bst_out* out) {
    if (!ctx || !a || !b || !out || (n_a > 0 && !a_legs) || (n_b > 0 && !b_legs)) {
        set_error("tk_contract_pairwise_f64: null argument");
        return TK_ERR_INVALID_ARG;
    }
    std::memset(out, 0, sizeof(*out));
    if (n_a != n_b || n_a < 1) {
        set_error("tk_contract_pairwise_f64: the operands must contract the same number (>= 1) of legs");
        return TK_ERR_INVALID_ARG;
    }
    std::string err;
    BstN A, B;
    if (!bstn_from_abi(*a, A, "A", err) || !bstn_from_abi(*b, B, "B", err)) {
        set_error("tk_contract_pairwise_f64: " + err);
        return TK_ERR_INVALID_ARG;
    }
    if (A.kind != B.kind) {
        set_error("tk_contract_pairwise_f64: quantum-number kinds differ");
        return TK_ERR_INVALID_ARG;
    }
    Fused2 FA, FB;
    BlockGemmPlan P;
    tk_status st = guard_host("tk_contract_pairwise_f64", err, [&]() -> tk_status {
        tk_status s2 = reshape_for_gemm(A, std::vector<int>(a_legs, a_legs + n_a), true, FA, err);
        if (s2 != TK_OK) return s2;
        if ((s2 = reshape_for_gemm(B, std::vector<int>(b_legs, b_legs + n_b), false, FB, err)) != TK_OK) return s2;
        return block_gemm_plan(FA.m, FB.m, P, err);
    });
    if (st != TK_OK) {
        set_error("tk_contract_pairwise_f64: " + err);
        return st;
    }
    // output header: fused legs owned by the output
    const int nc = qn_ncomp(A.kind);
    const QIndex* ol[2] = {&FA.m.legs[0], &FB.m.legs[1]};
    const size_t ns = (size_t)ol[0]->n() + ol[1]->n();
    out->owned_charges = (int32_t*)std::malloc(sizeof(int32_t) * std::max<size_t>(ns * nc, 1));
    out->owned_dims = (int64_t*)std::malloc(sizeof(int64_t) * std::max<size_t>(ns, 1));
    out->keys = (uint64_t*)std::malloc(sizeof(uint64_t) * std::max<size_t>(P.okeys.size(), 1));
    out->block_offsets = (int64_t*)std::malloc(sizeof(int64_t) * std::max<size_t>(P.ooffs.size(), 1));
    out->data = (double*)std::malloc(sizeof(double) * (size_t)std::max<int64_t>(P.total, 1));
    if (!out->owned_charges || !out->owned_dims || !out->keys || !out->block_offsets || !out->data) {
        tk_bst_free(out);
        set_error("tk_contract_pairwise_f64: host allocation failed");
        return TK_ERR_OOM;
    }
    size_t at = 0;
    for (int l = 0; l < 2; ++l) {
        out->legs[l].n_sectors = ol[l]->n();
        out->legs[l].charges = out->owned_charges + at * nc;
        out->legs[l].dims = out->owned_dims + at;
        for (int s = 0; s < ol[l]->n(); ++s, ++at) {
            for (int k = 0; k < nc; ++k) out->owned_charges[at * nc + k] = ol[l]->q[s].c[k];
            out->owned_dims[at] = ol[l]->dim[s];
        }
    }
    out->qn_kind = A.kind;
    out->rank = 2;
    out->leg_dirs[0] = FA.m.dirs[0];
    out->leg_dirs[1] = FB.m.dirs[1];
    out->flux[0] = P.target.c[0];
    out->flux[1] = P.target.c[1];
    out->n_blocks = (int64_t)P.okeys.size();
    out->total = P.total;
    std::copy(P.okeys.begin(), P.okeys.end(), out->keys);
    std::copy(P.ooffs.begin(), P.ooffs.end(), out->block_offsets);
    if (P.total == 0) return TK_OK;
    // device work: sources and tables in, fused operands gathered, GEMM, result out
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    struct Restore {
        int d;
        ~Restore() {
            if (d >= 0) cudaSetDevice(d);
        }
    } restore{prev};
    auto run = [&]() -> tk_status {
        CKC(cudaSetDevice(ctx->device));
        Blob blob;
        const size_t oa = blob.add(A.data, sizeof(double) * (size_t)A.total);
        const size_t ob = blob.add(B.data, sizeof(double) * (size_t)B.total);
        const size_t opa = blob.add(FA.pieces.data(), sizeof(FusePiece) * FA.pieces.size());
        const size_t opb = blob.add(FB.pieces.data(), sizeof(FusePiece) * FB.pieces.size());
        const size_t ot = blob.add(P.g.tasks.data(), sizeof(GemmTask) * P.g.tasks.size());
        const size_t og = blob.add(P.g.segs.data(), sizeof(GemmSeg) * P.g.segs.size());
        const size_t ol2 = blob.add(P.g.tiles.data(), sizeof(GemmTile) * P.g.tiles.size());
        // the fused operands and the result live on the device only, after the packed bytes
        const size_t dev_fa = (blob.size() + 255) & ~(size_t)255;
        const size_t dev_fb = (dev_fa + sizeof(double) * (size_t)FA.m.total + 255) & ~(size_t)255;
        const size_t dev_c = (dev_fb + sizeof(double) * (size_t)FB.m.total + 255) & ~(size_t)255;
        blob.tail = dev_c + sizeof(double) * (size_t)P.total;
        void* sp = nullptr;
        tk_status s2;
        if ((s2 = ctx_stream(ctx, &sp)) != TK_OK) return s2;
        cudaStream_t s = (cudaStream_t)sp;
        void *dv = nullptr, *hv = nullptr;
        if ((s2 = ctx_dev_scratch(ctx, blob.device_size(), &dv)) != TK_OK) return s2;
        if ((s2 = ctx_host_stage(ctx, std::max(blob.size(), sizeof(double) * (size_t)P.total), &hv)) != TK_OK)
            return s2;
        unsigned char* d = static_cast<unsigned char*>(dv);
        blob.copy_to(hv);
        CKC(cudaMemcpyAsync(d, hv, blob.size(), cudaMemcpyHostToDevice, s));
        double* fa = (double*)(d + dev_fa);
        double* fb = (double*)(d + dev_fb);
        // blocks of a fused tensor that no source block reaches are zero
        CKC(cudaMemsetAsync(fa, 0, sizeof(double) * (size_t)FA.m.total, s));
        CKC(cudaMemsetAsync(fb, 0, sizeof(double) * (size_t)FB.m.total, s));
        auto gather = [&](const Fused2& F, size_t opieces, size_t osrc, double* dst) -> cudaError_t {
            if (F.pieces.empty()) return cudaSuccess;
            int64_t maxel = 1;
            for (const FusePiece& p : F.pieces) maxel = std::max<int64_t>(maxel, (int64_t)p.rows * p.cols);
            dim3 grid((unsigned)std::min<int64_t>((maxel + 255) / 256, 64), (unsigned)F.pieces.size());
            fuse_gather_kernel<<<grid, 256, 0, s>>>((const FusePiece*)(d + opieces), (const double*)(d + osrc), dst);
            return cudaGetLastError();
        };
        if (FA.pieces.size() > 65535 || FB.pieces.size() > 65535) {
            set_error("tk_contract_pairwise_f64: more than 65535 blocks in one operand");
            return TK_ERR_UNSUPPORTED;
        }
        CKC(gather(FA, opa, oa, fa));
        CKC(gather(FB, opb, ob, fb));
        CKC(launch_gemm_f64((const GemmTile*)(d + ol2), (int)P.g.tiles.size(), (const GemmTask*)(d + ot),
                            (const GemmSeg*)(d + og), fa, fb, (double*)(d + dev_c), s));
        CKC(cudaMemcpyAsync(ctx->host_stage, d + dev_c, sizeof(double) * (size_t)P.total, cudaMemcpyDeviceToHost, s));
        CKC(cudaStreamSynchronize(s));
        std::memcpy(out->data, ctx->host_stage, sizeof(double) * (size_t)P.total);
        return TK_OK;
    };
    st = run();
    if (st != TK_OK) tk_bst_free(out);
    return st;
}
