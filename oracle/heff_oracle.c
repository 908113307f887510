/*
 * heff_oracle.c -- CPU restatement of tensorkraft's two-site H_eff path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * library and the timed CPU baseline.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it; the product never does.
 *
 * Parity status: the integer sector bookkeeping is pinned to the reference's
 * own known-answer tests (tests/golden/).  The H_eff matvec itself is
 * pinned by (a) a literal transliteration of the reference's dense builder,
 * (b) physics known answers (two-site Heisenberg spectrum, exact
 * diagonalisation of small chains).  The reference is a Rust workspace and
 * no Rust toolchain exists on the build machines, so its matvec could not be
 * run to produce golden vectors: matvec parity against reference-run
 * outputs is UNPINNED.
 *
 * Reference files restated here (paths inside kyungminlee/tensorkraft-design):
 *   tk-symmetry/src/builtins.rs:12-152     quantum-number packing (U1, Z2, U1Z2, U1Wide)
 *   tk-symmetry/src/sector_key.rs:31-55    PackedSectorKey::pack / unpack
 *   tk-symmetry/src/sector_key.rs:131-148  QIndex::offset_of / dim_of (linear scan)
 *   tk-symmetry/src/flux.rs:9-27           check_flux_rule
 *   tk-symmetry/src/flux.rs:43-234         enumerate_valid_sectors (DFS order)
 *   tk-dmrg/src/environments/mod.rs:92-95  Environment::get, layout (bra, w, ket)
 *   tk-dmrg/src/environments/mod.rs:491-602 build_heff_two_site + dense matvec closure
 * The U(1)xU(1) (N, 2Sz) type is new: the reference has no such type.  It
 * follows the reference's BitPackable pattern with 8 bits per component
 * (component 0 in the low byte), 16 bits per leg.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { ORC_U1 = 1, ORC_Z2 = 2, ORC_U1Z2 = 3, ORC_U1WIDE = 4, ORC_U1U1 = 5 };

typedef struct {
    int32_t n_sectors;
    const int32_t* charges; /* n_sectors * ncomp, sorted by the QN order */
    const int64_t* dims;    /* n_sectors */
} orc_qindex;

typedef struct {
    int32_t kind;
    int32_t rank;
    const orc_qindex* legs;  /* rank */
    int64_t n_blocks;
    const uint64_t* keys;    /* ascending */
    const int64_t* offsets;  /* start of each block in data */
    const double* data;      /* blocks back to back, each row-major */
} orc_bst;

/* ------------------------------------------------------------------ */
/* Quantum numbers (builtins.rs:12-152)                                */
/* ------------------------------------------------------------------ */

int orc_qn_ncomp(int kind) {
    return (kind == ORC_U1Z2 || kind == ORC_U1U1) ? 2 : 1;
}

int orc_qn_bits(int kind) {
    switch (kind) {
    case ORC_U1: return 8;
    case ORC_Z2: return 1;
    case ORC_U1Z2: return 9;
    case ORC_U1WIDE: return 16;
    case ORC_U1U1: return 16;
    default: return -1;
    }
}

static int32_t sext8(uint64_t v) { v &= 0xFF; return v >= 128 ? (int32_t)v - 256 : (int32_t)v; }
static int32_t sext16(uint64_t v) { v &= 0xFFFF; return v >= 32768 ? (int32_t)v - 65536 : (int32_t)v; }

/* BitPackable::pack: `(self.0 as u8) as u64` truncates to the low byte. */
uint64_t orc_qn_pack(int kind, const int32_t* q) {
    switch (kind) {
    case ORC_U1: return (uint64_t)((uint32_t)q[0] & 0xFFu);
    case ORC_Z2: return (uint64_t)(q[0] != 0);
    case ORC_U1Z2: return ((uint64_t)((uint32_t)q[0] & 0xFFu)) | ((uint64_t)(q[1] != 0) << 8);
    case ORC_U1WIDE: return (uint64_t)((uint32_t)q[0] & 0xFFFFu);
    case ORC_U1U1: return ((uint64_t)((uint32_t)q[0] & 0xFFu)) | ((uint64_t)((uint32_t)q[1] & 0xFFu) << 8);
    default: return 0;
    }
}

void orc_qn_unpack(int kind, uint64_t bits, int32_t* q) {
    switch (kind) {
    case ORC_U1: q[0] = sext8(bits); break;
    case ORC_Z2: q[0] = (int32_t)(bits & 1); break;
    case ORC_U1Z2: q[0] = sext8(bits); q[1] = (int32_t)((bits >> 8) & 1); break;
    case ORC_U1WIDE: q[0] = sext16(bits); break;
    case ORC_U1U1: q[0] = sext8(bits); q[1] = sext8(bits >> 8); break;
    default: break;
    }
}

/* fuse: U(1) components add, Z2 components xor. */
static void qn_fuse(int kind, const int32_t* a, const int32_t* b, int32_t* out) {
    switch (kind) {
    case ORC_Z2: out[0] = a[0] ^ b[0]; break;
    case ORC_U1Z2: out[0] = a[0] + b[0]; out[1] = a[1] ^ b[1]; break;
    case ORC_U1U1: out[0] = a[0] + b[0]; out[1] = a[1] + b[1]; break;
    default: out[0] = a[0] + b[0]; break;
    }
}

static void qn_dual(int kind, const int32_t* a, int32_t* out) {
    switch (kind) {
    case ORC_Z2: out[0] = a[0]; break;
    case ORC_U1Z2: out[0] = -a[0]; out[1] = a[1]; break;
    case ORC_U1U1: out[0] = -a[0]; out[1] = -a[1]; break;
    default: out[0] = -a[0]; break;
    }
}

static int qn_eq(int kind, const int32_t* a, const int32_t* b) {
    int n = orc_qn_ncomp(kind);
    for (int i = 0; i < n; ++i) if (a[i] != b[i]) return 0;
    return 1;
}

/* PackedSectorKey::pack (sector_key.rs:31-46): leg i at bits i*BIT_WIDTH. */
uint64_t orc_key_pack(int kind, int rank, const int32_t* qns) {
    int bw = orc_qn_bits(kind), nc = orc_qn_ncomp(kind);
    if (bw <= 0 || rank * bw > 64) return ~(uint64_t)0;
    uint64_t mask = (bw == 64) ? ~(uint64_t)0 : (((uint64_t)1 << bw) - 1);
    uint64_t key = 0;
    for (int i = 0; i < rank; ++i) key |= (orc_qn_pack(kind, qns + i * nc) & mask) << (i * bw);
    return key;
}

void orc_key_unpack(int kind, int rank, uint64_t key, int32_t* qns) {
    int bw = orc_qn_bits(kind), nc = orc_qn_ncomp(kind);
    uint64_t mask = ((uint64_t)1 << bw) - 1;
    for (int i = 0; i < rank; ++i) orc_qn_unpack(kind, (key >> (i * bw)) & mask, qns + i * nc);
}

/* check_flux_rule (flux.rs:9-27): Incoming legs fuse q, Outgoing legs fuse dual(q). */
int orc_check_flux_rule(int kind, int rank, const int32_t* qns, const int32_t* flux, const int8_t* dirs) {
    int nc = orc_qn_ncomp(kind);
    int32_t acc[2] = {0, 0}, t[2], d[2];
    for (int i = 0; i < rank; ++i) {
        if (dirs[i] == 0) { qn_fuse(kind, acc, qns + i * nc, t); }
        else { qn_dual(kind, qns + i * nc, d); qn_fuse(kind, acc, d, t); }
        acc[0] = t[0]; acc[1] = t[1];
    }
    return qn_eq(kind, acc, flux);
}

/* QIndex::offset_of / dim_of (sector_key.rs:131-148): linear scan. */
static int64_t qindex_find(int kind, const orc_qindex* ix, const int32_t* q, int64_t* offset) {
    int nc = orc_qn_ncomp(kind);
    int64_t off = 0;
    for (int32_t s = 0; s < ix->n_sectors; ++s) {
        if (qn_eq(kind, ix->charges + s * nc, q)) { if (offset) *offset = off; return s; }
        off += ix->dims[s];
    }
    return -1;
}

static int64_t qindex_total(const orc_qindex* ix) {
    int64_t t = 0;
    for (int32_t s = 0; s < ix->n_sectors; ++s) t += ix->dims[s];
    return t;
}

/*
 * enumerate_valid_sectors (flux.rs:43-234).  Depth-first over legs in QIndex
 * order; the last leg's charge is solved from the flux rule.  The reference's
 * memoised branch for rank > 4 only prunes subtrees that hold no result, so
 * both branches emit the same tuples in the same order, which this single
 * routine reproduces.  Output: sector indices per leg, `rank` int32 each.
 */
typedef struct {
    int kind, rank, nc;
    const orc_qindex* legs;
    const int32_t* flux;
    const int8_t* dirs;
    int32_t* out;
    int64_t cap, count;
    int32_t cur_idx[16];
    int32_t cur_q[32];
} enum_ctx;

static void enum_rec(enum_ctx* c, int depth) {
    int nc = c->nc;
    if (depth == c->rank - 1) {
        int32_t acc[2] = {0, 0}, t[2], d[2], req[2];
        for (int i = 0; i < depth; ++i) {
            if (c->dirs[i] == 0) qn_fuse(c->kind, acc, c->cur_q + i * nc, t);
            else { qn_dual(c->kind, c->cur_q + i * nc, d); qn_fuse(c->kind, acc, d, t); }
            acc[0] = t[0]; acc[1] = t[1];
        }
        qn_dual(c->kind, acc, d);
        qn_fuse(c->kind, c->flux, d, req);           /* flux (+) dual(partial) */
        if (c->dirs[depth] != 0) { qn_dual(c->kind, req, t); req[0] = t[0]; req[1] = t[1]; }
        int64_t s = qindex_find(c->kind, &c->legs[depth], req, NULL);
        if (s >= 0) {
            if (c->count < c->cap && c->out) {
                for (int i = 0; i < depth; ++i) c->out[c->count * c->rank + i] = c->cur_idx[i];
                c->out[c->count * c->rank + depth] = (int32_t)s;
            }
            c->count++;
        }
        return;
    }
    const orc_qindex* ix = &c->legs[depth];
    for (int32_t s = 0; s < ix->n_sectors; ++s) {
        c->cur_idx[depth] = s;
        for (int k = 0; k < nc; ++k) c->cur_q[depth * nc + k] = ix->charges[s * nc + k];
        enum_rec(c, depth + 1);
    }
}

int64_t orc_enumerate_valid_sectors(int kind, int rank, const orc_qindex* legs, const int32_t* flux,
                                    const int8_t* dirs, int32_t* out, int64_t cap) {
    if (rank < 1 || rank > 16) return -1;
    enum_ctx c;
    memset(&c, 0, sizeof c);
    c.kind = kind; c.rank = rank; c.nc = orc_qn_ncomp(kind);
    c.legs = legs; c.flux = flux; c.dirs = dirs; c.out = out; c.cap = cap;
    enum_rec(&c, 0);
    return c.count;
}

/* ------------------------------------------------------------------ */
/* Literal dense H_eff (environments/mod.rs:491-602)                   */
/* ------------------------------------------------------------------ */

static void block_qns_dims(const orc_bst* t, int64_t b, int32_t* qns, int64_t* dims, int64_t* offs) {
    int nc = orc_qn_ncomp(t->kind);
    orc_key_unpack(t->kind, t->rank, t->keys[b], qns);
    for (int l = 0; l < t->rank; ++l) {
        int64_t off = 0;
        int64_t s = qindex_find(t->kind, &t->legs[l], qns + l * nc, &off);
        dims[l] = s >= 0 ? t->legs[l].dims[s] : 0;
        offs[l] = s >= 0 ? off : 0; /* `.unwrap_or(0)` */
    }
}

/*
 * Builds the dense dim x dim matrix exactly as build_heff_two_site does:
 * MPO blocks of site i outer, site j inner (key order), w_mid paired by
 * quantum-number equality and block-local index, the 11-deep loop order of
 * :540-578, and the `in_idx < dim && out_idx < dim` guard of :574.
 * L and R are dense (bra, w, ket) row-major with bra dim == ket dim.
 */
int orc_heff_dense_build(const orc_bst* wi, const orc_bst* wj,
                         int64_t d_l, int64_t wl_tot, const double* L,
                         int64_t d_r, int64_t wr_tot, const double* R,
                         double* H) {
    int nc = orc_qn_ncomp(wi->kind);
    int64_t d_i = qindex_total(&wi->legs[0]);
    int64_t d_j = qindex_total(&wj->legs[0]);
    int64_t dim = d_i * d_j * d_l * d_r;
    memset(H, 0, sizeof(double) * (size_t)(dim * dim));
    int32_t qi[8], qj[8];
    int64_t di[4], dj[4], oi[4], oj[4];
    for (int64_t bi = 0; bi < wi->n_blocks; ++bi) {
        block_qns_dims(wi, bi, qi, di, oi);
        const double* mi = wi->data + wi->offsets[bi];
        for (int64_t bj = 0; bj < wj->n_blocks; ++bj) {
            block_qns_dims(wj, bj, qj, dj, oj);
            if (!qn_eq(wi->kind, qi + 3 * nc, qj + 2 * nc)) continue;
            const double* mj = wj->data + wj->offsets[bj];
            int64_t wm_n = di[3] < dj[2] ? di[3] : dj[2];
            for (int64_t sii = 0; sii < di[0]; ++sii)
            for (int64_t soi = 0; soi < di[1]; ++soi)
            for (int64_t sij = 0; sij < dj[0]; ++sij)
            for (int64_t soj = 0; soj < dj[1]; ++soj)
            for (int64_t wl = 0; wl < di[2]; ++wl)
            for (int64_t wm = 0; wm < wm_n; ++wm) {
                double wi_val = mi[sii * di[1] * di[2] * di[3] + soi * di[2] * di[3] + wl * di[3] + wm];
                for (int64_t wr = 0; wr < dj[3]; ++wr) {
                    double wj_val = mj[sij * dj[1] * dj[2] * dj[3] + soj * dj[2] * dj[3] + wm * dj[3] + wr];
                    double w_contrib = wi_val * wj_val;
                    for (int64_t a_l = 0; a_l < d_l; ++a_l)
                    for (int64_t ap_l = 0; ap_l < d_l; ++ap_l) {
                        double l_val = L[ap_l * wl_tot * d_l + (oi[2] + wl) * d_l + a_l];
                        double lw = l_val * w_contrib;
                        for (int64_t a_r = 0; a_r < d_r; ++a_r)
                        for (int64_t ap_r = 0; ap_r < d_r; ++ap_r) {
                            double r_val = R[ap_r * wr_tot * d_r + (oj[3] + wr) * d_r + a_r];
                            int64_t in_idx = (oi[0] + sii) * d_j * d_l * d_r + (oj[0] + sij) * d_l * d_r + a_l * d_r + a_r;
                            int64_t out_idx = (oi[1] + soi) * d_j * d_l * d_r + (oj[1] + soj) * d_l * d_r + ap_l * d_r + ap_r;
                            if (in_idx < dim && out_idx < dim) H[out_idx * dim + in_idx] += lw * r_val;
                        }
                    }
                }
            }
        }
    }
    return 0;
}

/* The closure of :592-599: y[i] = sum_j H[i*dim+j] * x[j]. */
void orc_dense_matvec(int64_t dim, const double* H, const double* x, double* y) {
    for (int64_t i = 0; i < dim; ++i) {
        double acc = 0.0;
        for (int64_t j = 0; j < dim; ++j) acc += H[i * dim + j] * x[j];
        y[i] = acc;
    }
}

/* ------------------------------------------------------------------ */
/* Dense factored matvec                                               */
/* ------------------------------------------------------------------ */

/*
 * Same sum as the dense builder, evaluated in the factored order
 * L -> W_i -> W_j -> R over the dense layouts (no sector tables at all):
 *   y[s'i,s'j,a',b'] = sum L[a',wl,a] Wi[si,s'i,wl,wm] Wj[sj,s'j,wm,wr]
 *                          R[b',wr,b] x[si,sj,a,b]
 * Wi is dense (d_i, d_i, wl, wm), Wj dense (d_j, d_j, wm, wr), global indices.
 */
int orc_heff_apply_dense(int64_t d_i, int64_t d_j, int64_t nwl, int64_t nwm, int64_t nwr,
                         const double* Wi, const double* Wj,
                         int64_t d_l, const double* L, int64_t d_r, const double* R,
                         const double* x, double* y) {
    int64_t P = d_i * d_j;
    int64_t DD = d_l * d_r;
    double* Wij = (double*)calloc((size_t)(P * P * nwl * nwr), sizeof(double));
    double* T1 = (double*)calloc((size_t)(P * nwl * DD), sizeof(double));
    double* T2 = (double*)calloc((size_t)(P * nwr * DD), sizeof(double));
    if (!Wij || !T1 || !T2) { free(Wij); free(T1); free(T2); return -1; }
    /* Wij[(si,sj),(s'i,s'j),wl,wr] = sum_wm Wi[si,s'i,wl,wm] Wj[sj,s'j,wm,wr] */
    for (int64_t si = 0; si < d_i; ++si) for (int64_t so = 0; so < d_i; ++so)
    for (int64_t sj = 0; sj < d_j; ++sj) for (int64_t to = 0; to < d_j; ++to)
    for (int64_t wl = 0; wl < nwl; ++wl) for (int64_t wr = 0; wr < nwr; ++wr) {
        double acc = 0.0;
        for (int64_t wm = 0; wm < nwm; ++wm)
            acc += Wi[((si * d_i + so) * nwl + wl) * nwm + wm] * Wj[((sj * d_j + to) * nwm + wm) * nwr + wr];
        Wij[(((si * d_j + sj) * P + (so * d_j + to)) * nwl + wl) * nwr + wr] = acc;
    }
    /* T1[p,wl,a',b] = sum_a L[a',wl,a] x[p,a,b] */
    #pragma omp parallel for collapse(2) schedule(static)
    for (int64_t p = 0; p < P; ++p)
    for (int64_t wl = 0; wl < nwl; ++wl) {
        double* t = T1 + (p * nwl + wl) * DD;
        const double* xp = x + p * DD;
        for (int64_t ap = 0; ap < d_l; ++ap)
        for (int64_t a = 0; a < d_l; ++a) {
            double lv = L[(ap * nwl + wl) * d_l + a];
            if (lv == 0.0) continue;
            for (int64_t b = 0; b < d_r; ++b) t[ap * d_r + b] += lv * xp[a * d_r + b];
        }
    }
    /* T2[p',wr,a',b] = sum_{p,wl} Wij[p,p',wl,wr] T1[p,wl,a',b] */
    #pragma omp parallel for collapse(2) schedule(static)
    for (int64_t po = 0; po < P; ++po)
    for (int64_t wr = 0; wr < nwr; ++wr) {
        double* t2 = T2 + (po * nwr + wr) * DD;
        for (int64_t p = 0; p < P; ++p)
        for (int64_t wl = 0; wl < nwl; ++wl) {
            double c = Wij[((p * P + po) * nwl + wl) * nwr + wr];
            if (c == 0.0) continue;
            const double* t1 = T1 + (p * nwl + wl) * DD;
            for (int64_t k = 0; k < DD; ++k) t2[k] += c * t1[k];
        }
    }
    /* y[p',a',b'] = sum_{wr,b} T2[p',wr,a',b] R[b',wr,b] */
    #pragma omp parallel for collapse(2) schedule(static)
    for (int64_t po = 0; po < P; ++po)
    for (int64_t ap = 0; ap < d_l; ++ap) {
        double* yr = y + po * DD + ap * d_r;
        for (int64_t bp = 0; bp < d_r; ++bp) yr[bp] = 0.0;
        for (int64_t wr = 0; wr < nwr; ++wr) {
            const double* t2 = T2 + (po * nwr + wr) * DD + ap * d_r;
            for (int64_t bp = 0; bp < d_r; ++bp) {
                const double* rr = R + (bp * nwr + wr) * d_r;
                double acc = 0.0;
                for (int64_t b = 0; b < d_r; ++b) acc += t2[b] * rr[b];
                yr[bp] += acc;
            }
        }
    }
    free(Wij); free(T1); free(T2);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Block-sparse matvec (the timed CPU baseline)                         */
/* ------------------------------------------------------------------ */

/*
 * A block-sparse restatement of the same contraction.  Sector structure:
 *   - psi blocks: enumerate_valid_sectors over legs (phys_i, phys_j, alpha_L,
 *     alpha_R) with directions (In, In, In, Out) and the given flux, stored
 *     in ascending packed-key order (BlockSparseTensor::zeros,
 *     block_sparse.rs:40-84), each block row-major (phys_i, phys_j, aL, aR)
 *     and the blocks back to back (FlatBlockStorage, flat_storage.rs:95-130).
 *     flux == NULL selects every sector combination.
 *   - L/R blocks: a (bra sector, channel, ket sector) slab takes part when
 *     any of its entries is non-zero (zero slabs add nothing to the sum).
 * Work is split into sector GEMM tasks run in descending-cost order (LPT,
 * tk-linalg/src/tasks.rs:172-174) over OpenMP threads.
 */
typedef struct {
    int kind, nc;
    int64_t d_i, d_j, nwl, nwr, d_l, d_r;
    int32_t nA, nB, nSi, nSj;
    int64_t *offA, *dimA, *offB, *dimB;
    int32_t *secI, *secJ;          /* physical state -> sector */
    int64_t *locI, *locJ;          /* physical state -> index inside its sector */
    int64_t *dimSi, *dimSj;
    /* psi blocks */
    int64_t n_blocks;
    int32_t* blk;                  /* n_blocks * 4 sector indices */
    int64_t* blk_off;              /* element offset of each block */
    int64_t total;
    int64_t* blk_of;               /* [nSi][nSj][nA][nB] -> block index or -1 */
    /* nonzero slabs */
    uint8_t* Lnz;                  /* [nA][nwl][nA] */
    uint8_t* Rnz;                  /* [nB][nwr][nB] */
    double* RT;                    /* R transposed per slab: [wr][b][b'] (dense d_r x d_r per wr) */
    double* Wij;                   /* [p][p'][wl][wr] */
    int64_t P;
    /* T1 / T2 tables */
    int64_t* t1_off;               /* [P][nwl][nA][nB] -> offset or -1 */
    int64_t t1_total;
    int64_t* t2_off;               /* [P][nwr][nA][nB] */
    int64_t t2_total;
    /* the non-empty tasks of each step, in descending-cost (LPT) order */
    struct orc_task *task1, *task2, *task3;
    int64_t n_task1, n_task2, n_task3;
    double* T1;
    double* T2;
    const double* L;
    const double* R;
} orc_bs_plan;

static int64_t q_total(const orc_qindex* ix) { return qindex_total(ix); }

static void state_maps(const orc_qindex* ix, int32_t* sec, int64_t* loc) {
    int64_t s = 0;
    for (int32_t k = 0; k < ix->n_sectors; ++k)
        for (int64_t i = 0; i < ix->dims[k]; ++i) { sec[s] = k; loc[s] = i; ++s; }
}

typedef struct { uint64_t key; int32_t idx[4]; } keyed4;
static int cmp_keyed4(const void* a, const void* b) {
    uint64_t x = ((const keyed4*)a)->key, y = ((const keyed4*)b)->key;
    return x < y ? -1 : (x > y ? 1 : 0);
}

void orc_bs_destroy(orc_bs_plan* p);
static int build_tasks(orc_bs_plan* p);

/* psi_flux may be NULL (all sectors). */
orc_bs_plan* orc_bs_create(int kind, const orc_qindex* phys_i, const orc_qindex* phys_j,
                           const orc_qindex* alpha_l, const orc_qindex* alpha_r,
                           const int32_t* psi_flux,
                           int64_t nwl, int64_t nwm, int64_t nwr,
                           const double* Wi, const double* Wj,
                           const double* L, const double* R) {
    orc_bs_plan* p = (orc_bs_plan*)calloc(1, sizeof(orc_bs_plan));
    if (!p) return NULL;
    p->kind = kind; p->nc = orc_qn_ncomp(kind);
    p->d_i = q_total(phys_i); p->d_j = q_total(phys_j);
    p->d_l = q_total(alpha_l); p->d_r = q_total(alpha_r);
    p->nwl = nwl; p->nwr = nwr;
    p->nA = alpha_l->n_sectors; p->nB = alpha_r->n_sectors;
    p->nSi = phys_i->n_sectors; p->nSj = phys_j->n_sectors;
    p->L = L; p->R = R;
    p->P = p->d_i * p->d_j;
    int32_t nA = p->nA, nB = p->nB;
    p->offA = (int64_t*)malloc(sizeof(int64_t) * nA); p->dimA = (int64_t*)malloc(sizeof(int64_t) * nA);
    p->offB = (int64_t*)malloc(sizeof(int64_t) * nB); p->dimB = (int64_t*)malloc(sizeof(int64_t) * nB);
    { int64_t o = 0; for (int32_t a = 0; a < nA; ++a) { p->offA[a] = o; p->dimA[a] = alpha_l->dims[a]; o += alpha_l->dims[a]; } }
    { int64_t o = 0; for (int32_t b = 0; b < nB; ++b) { p->offB[b] = o; p->dimB[b] = alpha_r->dims[b]; o += alpha_r->dims[b]; } }
    p->secI = (int32_t*)malloc(sizeof(int32_t) * p->d_i); p->locI = (int64_t*)malloc(sizeof(int64_t) * p->d_i);
    p->secJ = (int32_t*)malloc(sizeof(int32_t) * p->d_j); p->locJ = (int64_t*)malloc(sizeof(int64_t) * p->d_j);
    state_maps(phys_i, p->secI, p->locI);
    state_maps(phys_j, p->secJ, p->locJ);
    p->dimSi = (int64_t*)malloc(sizeof(int64_t) * p->nSi); p->dimSj = (int64_t*)malloc(sizeof(int64_t) * p->nSj);
    for (int32_t k = 0; k < p->nSi; ++k) p->dimSi[k] = phys_i->dims[k];
    for (int32_t k = 0; k < p->nSj; ++k) p->dimSj[k] = phys_j->dims[k];

    /* psi block list */
    orc_qindex legs[4] = {*phys_i, *phys_j, *alpha_l, *alpha_r};
    int8_t dirs[4] = {0, 0, 0, 1};
    int64_t cap;
    int32_t* tuples;
    if (psi_flux) {
        cap = orc_enumerate_valid_sectors(kind, 4, legs, psi_flux, dirs, NULL, 0);
        tuples = (int32_t*)malloc(sizeof(int32_t) * 4 * (cap > 0 ? cap : 1));
        orc_enumerate_valid_sectors(kind, 4, legs, psi_flux, dirs, tuples, cap);
    } else {
        cap = (int64_t)p->nSi * p->nSj * nA * nB;
        tuples = (int32_t*)malloc(sizeof(int32_t) * 4 * cap);
        int64_t n = 0;
        for (int32_t a = 0; a < p->nSi; ++a) for (int32_t b = 0; b < p->nSj; ++b)
        for (int32_t c = 0; c < nA; ++c) for (int32_t d = 0; d < nB; ++d) {
            tuples[n * 4 + 0] = a; tuples[n * 4 + 1] = b; tuples[n * 4 + 2] = c; tuples[n * 4 + 3] = d; ++n;
        }
    }
    keyed4* kb = (keyed4*)malloc(sizeof(keyed4) * (cap > 0 ? cap : 1));
    for (int64_t n = 0; n < cap; ++n) {
        int32_t q[8];
        for (int l = 0; l < 4; ++l)
            for (int k = 0; k < p->nc; ++k) q[l * p->nc + k] = legs[l].charges[tuples[n * 4 + l] * p->nc + k];
        kb[n].key = orc_key_pack(kind, 4, q);
        memcpy(kb[n].idx, tuples + n * 4, sizeof(int32_t) * 4);
    }
    qsort(kb, (size_t)cap, sizeof(keyed4), cmp_keyed4);
    p->n_blocks = cap;
    p->blk = (int32_t*)malloc(sizeof(int32_t) * 4 * (cap > 0 ? cap : 1));
    p->blk_off = (int64_t*)malloc(sizeof(int64_t) * (cap > 0 ? cap : 1));
    int64_t nsec = (int64_t)p->nSi * p->nSj * nA * nB;
    p->blk_of = (int64_t*)malloc(sizeof(int64_t) * nsec);
    for (int64_t i = 0; i < nsec; ++i) p->blk_of[i] = -1;
    int64_t off = 0;
    for (int64_t n = 0; n < cap; ++n) {
        memcpy(p->blk + n * 4, kb[n].idx, sizeof(int32_t) * 4);
        p->blk_off[n] = off;
        int32_t* t = kb[n].idx;
        p->blk_of[(((int64_t)t[0] * p->nSj + t[1]) * nA + t[2]) * nB + t[3]] = n;
        off += p->dimSi[t[0]] * p->dimSj[t[1]] * p->dimA[t[2]] * p->dimB[t[3]];
    }
    p->total = off;
    free(kb); free(tuples);

    /* non-zero slabs of L and R */
    p->Lnz = (uint8_t*)calloc((size_t)nA * nwl * nA, 1);
    for (int32_t ap = 0; ap < nA; ++ap) for (int64_t w = 0; w < nwl; ++w) for (int32_t a = 0; a < nA; ++a) {
        int nz = 0;
        for (int64_t i = 0; i < p->dimA[ap] && !nz; ++i)
            for (int64_t j = 0; j < p->dimA[a]; ++j)
                if (L[((p->offA[ap] + i) * nwl + w) * p->d_l + p->offA[a] + j] != 0.0) { nz = 1; break; }
        p->Lnz[((int64_t)ap * nwl + w) * nA + a] = (uint8_t)nz;
    }
    p->Rnz = (uint8_t*)calloc((size_t)nB * nwr * nB, 1);
    for (int32_t bp = 0; bp < nB; ++bp) for (int64_t w = 0; w < nwr; ++w) for (int32_t b = 0; b < nB; ++b) {
        int nz = 0;
        for (int64_t i = 0; i < p->dimB[bp] && !nz; ++i)
            for (int64_t j = 0; j < p->dimB[b]; ++j)
                if (R[((p->offB[bp] + i) * nwr + w) * p->d_r + p->offB[b] + j] != 0.0) { nz = 1; break; }
        p->Rnz[((int64_t)bp * nwr + w) * nB + b] = (uint8_t)nz;
    }
    /* R transposed per channel: RT[w][b][b'] = R[b'][w][b] */
    p->RT = (double*)malloc(sizeof(double) * (size_t)(nwr * p->d_r * p->d_r));
    for (int64_t w = 0; w < nwr; ++w) for (int64_t b = 0; b < p->d_r; ++b) for (int64_t bp = 0; bp < p->d_r; ++bp)
        p->RT[(w * p->d_r + b) * p->d_r + bp] = R[(bp * nwr + w) * p->d_r + b];

    /* two-site operator */
    int64_t P = p->P;
    p->Wij = (double*)calloc((size_t)(P * P * nwl * nwr), sizeof(double));
    for (int64_t si = 0; si < p->d_i; ++si) for (int64_t so = 0; so < p->d_i; ++so)
    for (int64_t sj = 0; sj < p->d_j; ++sj) for (int64_t to = 0; to < p->d_j; ++to)
    for (int64_t wl = 0; wl < nwl; ++wl) for (int64_t wr = 0; wr < nwr; ++wr) {
        double acc = 0.0;
        for (int64_t wm = 0; wm < nwm; ++wm)
            acc += Wi[((si * p->d_i + so) * nwl + wl) * nwm + wm] * Wj[((sj * p->d_j + to) * nwm + wm) * nwr + wr];
        p->Wij[(((si * p->d_j + sj) * P + (so * p->d_j + to)) * nwl + wl) * nwr + wr] = acc;
    }

    /* T1[p, wl, A', B] exists when some A has an L slab (A', wl, A) and a psi block (p, A, B). */
    int64_t n1 = P * nwl * nA * nB;
    p->t1_off = (int64_t*)malloc(sizeof(int64_t) * n1);
    off = 0;
    for (int64_t pp = 0; pp < P; ++pp) {
        int32_t si = p->secI[pp / p->d_j], sj = p->secJ[pp % p->d_j];
        for (int64_t wl = 0; wl < nwl; ++wl) for (int32_t ap = 0; ap < nA; ++ap) for (int32_t b = 0; b < nB; ++b) {
            int ex = 0;
            for (int32_t a = 0; a < nA && !ex; ++a)
                if (p->Lnz[((int64_t)ap * nwl + wl) * nA + a] &&
                    p->blk_of[(((int64_t)si * p->nSj + sj) * nA + a) * nB + b] >= 0) ex = 1;
            int64_t id = ((pp * nwl + wl) * nA + ap) * nB + b;
            if (ex) { p->t1_off[id] = off; off += p->dimA[ap] * p->dimB[b]; } else p->t1_off[id] = -1;
        }
    }
    p->t1_total = off;
    int64_t n2 = P * nwr * nA * nB;
    p->t2_off = (int64_t*)malloc(sizeof(int64_t) * n2);
    off = 0;
    for (int64_t po = 0; po < P; ++po) for (int64_t wr = 0; wr < nwr; ++wr)
    for (int32_t ap = 0; ap < nA; ++ap) for (int32_t b = 0; b < nB; ++b) {
        int ex = 0;
        for (int64_t pp = 0; pp < P && !ex; ++pp) for (int64_t wl = 0; wl < nwl; ++wl)
            if (p->Wij[((pp * P + po) * nwl + wl) * nwr + wr] != 0.0 &&
                p->t1_off[((pp * nwl + wl) * nA + ap) * nB + b] >= 0) { ex = 1; break; }
        int64_t id = ((po * nwr + wr) * nA + ap) * nB + b;
        if (ex) { p->t2_off[id] = off; off += p->dimA[ap] * p->dimB[b]; } else p->t2_off[id] = -1;
    }
    p->t2_total = off;
    p->T1 = (double*)malloc(sizeof(double) * (size_t)(p->t1_total > 0 ? p->t1_total : 1));
    p->T2 = (double*)malloc(sizeof(double) * (size_t)(p->t2_total > 0 ? p->t2_total : 1));
    if (!p->T1 || !p->T2 || build_tasks(p) != 0) { orc_bs_destroy(p); return NULL; }
    return p;
}

int64_t orc_bs_total(const orc_bs_plan* p) { return p->total; }
int64_t orc_bs_n_blocks(const orc_bs_plan* p) { return p->n_blocks; }
void orc_bs_blocks(const orc_bs_plan* p, int32_t* sectors, int64_t* offsets) {
    memcpy(sectors, p->blk, sizeof(int32_t) * 4 * p->n_blocks);
    memcpy(offsets, p->blk_off, sizeof(int64_t) * p->n_blocks);
}

void orc_bs_destroy(orc_bs_plan* p) {
    if (!p) return;
    free(p->offA); free(p->dimA); free(p->offB); free(p->dimB);
    free(p->secI); free(p->locI); free(p->secJ); free(p->locJ); free(p->dimSi); free(p->dimSj);
    free(p->blk); free(p->blk_off); free(p->blk_of); free(p->Lnz); free(p->Rnz); free(p->RT);
    free(p->Wij); free(p->t1_off); free(p->t2_off); free(p->T1); free(p->T2);
    free(p->task1); free(p->task2); free(p->task3);
    free(p);
}

/* Address of the (si, sj) state pair's aL x aR matrix inside its psi block. */
static int64_t psi_sub(const orc_bs_plan* p, int64_t pp, int32_t a, int32_t b) {
    int64_t si = pp / p->d_j, sj = pp % p->d_j;
    int32_t ki = p->secI[si], kj = p->secJ[sj];
    int64_t blk = p->blk_of[(((int64_t)ki * p->nSj + kj) * p->nA + a) * p->nB + b];
    if (blk < 0) return -1;
    int64_t sub = p->locI[si] * p->dimSj[kj] + p->locJ[sj];
    return p->blk_off[blk] + sub * p->dimA[a] * p->dimB[b];
}

/*
 * C[M x N] += A[M x K] B[K x N], row-major with leading dimensions lda, ldb,
 * ldc.  This is the plain i-k-j loop, register-blocked: 4 x 4 tiles of C
 * live in locals over panels of 256 k, so the 256 x 4 panel of B stays in L1
 * while the row tiles stream past it.  Every element of C still adds its
 * products one at a time in ascending k, which keeps the sums bit-identical
 * to the unblocked loop on every host (ISO C mode keeps the compiler from
 * contracting them into fused multiply-adds).  The per-task products of the
 * reference's block GEMM go to faer's matmul
 * (tk-linalg/src/device/faer.rs:475-482); this blocking stands in for that
 * library's cache blocking.
 */
enum { ORC_MR = 4, ORC_NR = 4, ORC_KB = 256 };

static void tile_mr(int64_t kb, const double* restrict A, int64_t lda, const double* restrict B, int64_t ldb,
                    double* restrict C, int64_t ldc) {
    double c[ORC_MR][ORC_NR];
    for (int i = 0; i < ORC_MR; ++i)
        for (int j = 0; j < ORC_NR; ++j) c[i][j] = C[i * ldc + j];
    for (int64_t k = 0; k < kb; ++k) {
        const double* b = B + k * ldb;
        for (int i = 0; i < ORC_MR; ++i) {
            const double a = A[i * lda + k];
            for (int j = 0; j < ORC_NR; ++j) c[i][j] += a * b[j];
        }
    }
    for (int i = 0; i < ORC_MR; ++i)
        for (int j = 0; j < ORC_NR; ++j) C[i * ldc + j] = c[i][j];
}

static void tile_1(int64_t kb, const double* restrict A, const double* restrict B, int64_t ldb, double* restrict C) {
    double c[ORC_NR];
    for (int j = 0; j < ORC_NR; ++j) c[j] = C[j];
    for (int64_t k = 0; k < kb; ++k) {
        const double* b = B + k * ldb;
        const double a = A[k];
        for (int j = 0; j < ORC_NR; ++j) c[j] += a * b[j];
    }
    for (int j = 0; j < ORC_NR; ++j) C[j] = c[j];
}

static void gemm_acc(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const double* B, int64_t ldb,
                     double* C, int64_t ldc) {
    for (int64_t k0 = 0; k0 < K; k0 += ORC_KB) {
        const int64_t kb = K - k0 < ORC_KB ? K - k0 : ORC_KB;
        int64_t j0 = 0;
        for (; j0 + ORC_NR <= N; j0 += ORC_NR) {
            int64_t i0 = 0;
            for (; i0 + ORC_MR <= M; i0 += ORC_MR)
                tile_mr(kb, A + i0 * lda + k0, lda, B + k0 * ldb + j0, ldb, C + i0 * ldc + j0, ldc);
            for (; i0 < M; ++i0) tile_1(kb, A + i0 * lda + k0, B + k0 * ldb + j0, ldb, C + i0 * ldc + j0);
        }
        if (j0 < N)
            for (int64_t i = 0; i < M; ++i) {
                double* c = C + i * ldc;
                for (int64_t k = k0; k < k0 + kb; ++k) {
                    const double a = A[i * lda + k];
                    const double* b = B + k * ldb;
                    for (int64_t j = j0; j < N; ++j) c[j] += a * b[j];
                }
            }
    }
}

/* Sector GEMM tasks of the three steps, ordered by descending cost (ties by
 * task id, then row) as the reference orders its block-GEMM tasks before
 * handing them to its thread pool (tk-linalg/src/tasks.rs:172-174).  Step-1
 * and step-3 tasks taller than ORC_ROWS rows are cut into row ranges, so a
 * few large sectors still spread over all threads; a row range computes its
 * rows exactly as the whole task would. */
enum { ORC_ROWS = 64 };

typedef struct orc_task { double cost; int64_t id; int32_t r0, r1; } orc_task;

typedef struct { orc_task* t; int64_t n, cap; } orc_task_list;

static int cmp_task(const void* a, const void* b) {
    const orc_task *x = (const orc_task*)a, *y = (const orc_task*)b;
    if (x->cost != y->cost) return x->cost > y->cost ? -1 : 1;
    if (x->id != y->id) return x->id < y->id ? -1 : 1;
    return x->r0 < y->r0 ? -1 : (x->r0 > y->r0 ? 1 : 0);
}

/* Appends the row ranges of one task of `rows` rows and total cost `cost`
 * (one range of every row when `split` is 0); returns -1 when out of memory. */
static int push_rows(orc_task_list* L, int64_t id, int64_t rows, double cost, int split) {
    const int64_t step = (split && rows > ORC_ROWS) ? ORC_ROWS : (rows > 0 ? rows : 1);
    const int64_t parts = rows > 0 ? (rows + step - 1) / step : 1;
    if (L->n + parts > L->cap) {
        int64_t cap = L->cap > 0 ? 2 * L->cap : 1024;
        while (cap < L->n + parts) cap *= 2;
        orc_task* t = (orc_task*)realloc(L->t, sizeof(orc_task) * (size_t)cap);
        if (!t) return -1;
        L->t = t;
        L->cap = cap;
    }
    for (int64_t k = 0; k < parts; ++k) {
        const int64_t r0 = k * step, r1 = r0 + step < rows ? r0 + step : rows;
        orc_task* e = L->t + L->n++;
        e->cost = rows > 0 ? cost * (double)(r1 - r0) / (double)rows : cost;
        e->id = id;
        e->r0 = (int32_t)r0;
        e->r1 = (int32_t)r1;
    }
    return 0;
}

/* Sorts the list in LPT order and hands its array to the caller. */
static orc_task* lpt_sorted(orc_task_list* L, int64_t* n) {
    if (!L->t) L->t = (orc_task*)malloc(sizeof(orc_task));
    if (L->t) qsort(L->t, (size_t)L->n, sizeof(orc_task), cmp_task);
    *n = L->n;
    orc_task* out = L->t;
    L->t = NULL;
    L->n = L->cap = 0;
    return out;
}

static int build_tasks(orc_bs_plan* p) {
    const int64_t P = p->P, nwl = p->nwl, nwr = p->nwr;
    const int32_t nA = p->nA, nB = p->nB;
    const int64_t n1 = P * nwl * nA * nB, n2 = P * nwr * nA * nB, n3 = P * nA * nB;
    orc_task_list L = {NULL, 0, 0};
    int err = 0;
    for (int64_t id = 0; id < n1 && !err; ++id) {
        if (p->t1_off[id] < 0) continue;
        const int32_t b = (int32_t)(id % nB), ap = (int32_t)((id / nB) % nA);
        const int64_t wl = (id / ((int64_t)nB * nA)) % nwl, pp = id / ((int64_t)nB * nA * nwl);
        double c = 0.0;
        for (int32_t a = 0; a < nA; ++a)
            if (p->Lnz[((int64_t)ap * nwl + wl) * nA + a] && psi_sub(p, pp, a, b) >= 0)
                c += (double)p->dimA[ap] * p->dimA[a] * p->dimB[b];
        err = push_rows(&L, id, p->dimA[ap], c, 1);
    }
    p->task1 = lpt_sorted(&L, &p->n_task1);
    for (int64_t id = 0; id < n2 && !err; ++id) {
        if (p->t2_off[id] < 0) continue;
        const int32_t b = (int32_t)(id % nB), ap = (int32_t)((id / nB) % nA);
        const int64_t wr = (id / ((int64_t)nB * nA)) % nwr, po = id / ((int64_t)nB * nA * nwr);
        double c = 0.0;
        for (int64_t pp = 0; pp < P; ++pp) for (int64_t wl = 0; wl < nwl; ++wl)
            if (p->Wij[((pp * P + po) * nwl + wl) * nwr + wr] != 0.0 &&
                p->t1_off[((pp * nwl + wl) * nA + ap) * nB + b] >= 0)
                c += (double)p->dimA[ap] * p->dimB[b];
        err = push_rows(&L, id, p->dimA[ap], c, 0);
    }
    p->task2 = lpt_sorted(&L, &p->n_task2);
    for (int64_t id = 0; id < n3 && !err; ++id) {
        const int32_t bp = (int32_t)(id % nB), ap = (int32_t)((id / nB) % nA);
        const int64_t po = id / ((int64_t)nB * nA);
        if (psi_sub(p, po, ap, bp) < 0) continue;
        double c = 0.0;
        for (int64_t wr = 0; wr < nwr; ++wr) for (int32_t b = 0; b < nB; ++b)
            if (p->Rnz[((int64_t)bp * nwr + wr) * nB + b] && p->t2_off[((po * nwr + wr) * nA + ap) * nB + b] >= 0)
                c += (double)p->dimA[ap] * p->dimB[bp] * p->dimB[b];
        err = push_rows(&L, id, p->dimA[ap], c, 1);
    }
    p->task3 = lpt_sorted(&L, &p->n_task3);
    free(L.t);
    return (!err && p->task1 && p->task2 && p->task3) ? 0 : -1;
}

/* x and y in the block layout; y fully overwritten. */
int orc_bs_apply(orc_bs_plan* p, const double* x, double* y) {
    const int64_t nwl = p->nwl, nwr = p->nwr;
    const int32_t nA = p->nA, nB = p->nB;
    /* step 1: T1[p,wl,A',B] = sum_A L[A',wl,A] x[p,A,B], rows r0..r1 of A' */
    #pragma omp parallel for schedule(dynamic, 1)
    for (int64_t t = 0; t < p->n_task1; ++t) {
        const orc_task* tk = p->task1 + t;
        const int64_t id = tk->id, r0 = tk->r0, M = tk->r1 - tk->r0;
        const int32_t b = (int32_t)(id % nB);
        const int32_t ap = (int32_t)((id / nB) % nA);
        const int64_t wl = (id / ((int64_t)nB * nA)) % nwl;
        const int64_t pp = id / ((int64_t)nB * nA * nwl);
        const int64_t N = p->dimB[b];
        double* t1 = p->T1 + p->t1_off[id] + r0 * N;
        memset(t1, 0, sizeof(double) * (size_t)(M * N));
        for (int32_t a = 0; a < nA; ++a) {
            if (!p->Lnz[((int64_t)ap * nwl + wl) * nA + a]) continue;
            const int64_t xo = psi_sub(p, pp, a, b);
            if (xo < 0) continue;
            const double* l = p->L + ((p->offA[ap] + r0) * nwl + wl) * p->d_l + p->offA[a];
            gemm_acc(M, N, p->dimA[a], l, nwl * p->d_l, x + xo, N, t1, N);
        }
    }
    /* step 2: T2[p',wr,A',B] = sum_{p,wl} Wij[p,p',wl,wr] T1[p,wl,A',B] */
    #pragma omp parallel for schedule(dynamic, 1)
    for (int64_t t = 0; t < p->n_task2; ++t) {
        const int64_t id = p->task2[t].id;
        const int32_t b = (int32_t)(id % nB);
        const int32_t ap = (int32_t)((id / nB) % nA);
        const int64_t wr = (id / ((int64_t)nB * nA)) % nwr;
        const int64_t po = id / ((int64_t)nB * nA * nwr);
        const int64_t MN = p->dimA[ap] * p->dimB[b];
        double* t2 = p->T2 + p->t2_off[id];
        memset(t2, 0, sizeof(double) * (size_t)MN);
        for (int64_t pp = 0; pp < p->P; ++pp) for (int64_t wl = 0; wl < nwl; ++wl) {
            const double c = p->Wij[((pp * p->P + po) * nwl + wl) * nwr + wr];
            if (c == 0.0) continue;
            const int64_t o1 = p->t1_off[((pp * nwl + wl) * nA + ap) * nB + b];
            if (o1 < 0) continue;
            const double* t1 = p->T1 + o1;
            for (int64_t k = 0; k < MN; ++k) t2[k] += c * t1[k];
        }
    }
    /* step 3: y[p',A',B'] = sum_{wr,B} T2[p',wr,A',B] R[B',wr,B], rows r0..r1 of A' */
    #pragma omp parallel for schedule(dynamic, 1)
    for (int64_t t = 0; t < p->n_task3; ++t) {
        const orc_task* tk = p->task3 + t;
        const int64_t id = tk->id, r0 = tk->r0, M = tk->r1 - tk->r0;
        const int32_t bp = (int32_t)(id % nB);
        const int32_t ap = (int32_t)((id / nB) % nA);
        const int64_t po = id / ((int64_t)nB * nA);
        const int64_t N = p->dimB[bp];
        double* ys = y + psi_sub(p, po, ap, bp) + r0 * N;
        memset(ys, 0, sizeof(double) * (size_t)(M * N));
        for (int64_t wr = 0; wr < nwr; ++wr) for (int32_t b = 0; b < nB; ++b) {
            if (!p->Rnz[((int64_t)bp * nwr + wr) * nB + b]) continue;
            const int64_t o2 = p->t2_off[((po * nwr + wr) * nA + ap) * nB + b];
            if (o2 < 0) continue;
            const int64_t K = p->dimB[b];
            gemm_acc(M, N, K, p->T2 + o2 + r0 * K, K, p->RT + (wr * p->d_r + p->offB[b]) * p->d_r + p->offB[bp],
                     p->d_r, ys, N);
        }
    }
    return 0;
}

/* Algorithmic flop count of one orc_bs_apply (2 flops per multiply-add). */
double orc_bs_flops(const orc_bs_plan* p) {
    double f = 0.0;
    int64_t P = p->P, nwl = p->nwl, nwr = p->nwr;
    int32_t nA = p->nA, nB = p->nB;
    for (int64_t pp = 0; pp < P; ++pp) for (int64_t wl = 0; wl < nwl; ++wl)
    for (int32_t ap = 0; ap < nA; ++ap) for (int32_t b = 0; b < nB; ++b) {
        if (p->t1_off[((pp * nwl + wl) * nA + ap) * nB + b] < 0) continue;
        for (int32_t a = 0; a < nA; ++a)
            if (p->Lnz[((int64_t)ap * nwl + wl) * nA + a] && psi_sub(p, pp, a, b) >= 0)
                f += 2.0 * p->dimA[ap] * p->dimA[a] * p->dimB[b];
    }
    for (int64_t po = 0; po < P; ++po) for (int64_t wr = 0; wr < nwr; ++wr)
    for (int32_t ap = 0; ap < nA; ++ap) for (int32_t b = 0; b < nB; ++b) {
        if (p->t2_off[((po * nwr + wr) * nA + ap) * nB + b] < 0) continue;
        for (int64_t pp = 0; pp < P; ++pp) for (int64_t wl = 0; wl < nwl; ++wl)
            if (p->Wij[((pp * P + po) * nwl + wl) * nwr + wr] != 0.0 &&
                p->t1_off[((pp * nwl + wl) * nA + ap) * nB + b] >= 0)
                f += 2.0 * p->dimA[ap] * p->dimB[b];
    }
    for (int64_t po = 0; po < P; ++po) for (int32_t ap = 0; ap < nA; ++ap) for (int32_t bp = 0; bp < nB; ++bp) {
        if (psi_sub(p, po, ap, bp) < 0) continue;
        for (int64_t wr = 0; wr < nwr; ++wr) for (int32_t b = 0; b < nB; ++b)
            if (p->Rnz[((int64_t)bp * nwr + wr) * nB + b] && p->t2_off[((po * nwr + wr) * nA + ap) * nB + b] >= 0)
                f += 2.0 * p->dimA[ap] * p->dimB[bp] * p->dimB[b];
    }
    return f;
}

/* Scatter/gather between the dense (si, sj, aL, aR) layout and the block layout. */
void orc_bs_to_dense(const orc_bs_plan* p, const double* xb, double* xd) {
    int64_t DD = p->d_l * p->d_r;
    memset(xd, 0, sizeof(double) * (size_t)(p->P * DD));
    for (int64_t pp = 0; pp < p->P; ++pp) for (int32_t a = 0; a < p->nA; ++a) for (int32_t b = 0; b < p->nB; ++b) {
        int64_t o = psi_sub(p, pp, a, b);
        if (o < 0) continue;
        for (int64_t i = 0; i < p->dimA[a]; ++i)
            memcpy(xd + pp * DD + (p->offA[a] + i) * p->d_r + p->offB[b], xb + o + i * p->dimB[b], sizeof(double) * (size_t)p->dimB[b]);
    }
}

void orc_bs_from_dense(const orc_bs_plan* p, const double* xd, double* xb) {
    int64_t DD = p->d_l * p->d_r;
    for (int64_t pp = 0; pp < p->P; ++pp) for (int32_t a = 0; a < p->nA; ++a) for (int32_t b = 0; b < p->nB; ++b) {
        int64_t o = psi_sub(p, pp, a, b);
        if (o < 0) continue;
        for (int64_t i = 0; i < p->dimA[a]; ++i)
            memcpy(xb + o + i * p->dimB[b], xd + pp * DD + (p->offA[a] + i) * p->d_r + p->offB[b], sizeof(double) * (size_t)p->dimB[b]);
    }
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}
