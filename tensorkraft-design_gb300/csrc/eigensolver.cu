// lanczos.cu -- device Lanczos for the lowest eigenpair of a two-site H_eff.
//
// Restates LanczosSolver::lowest_eigenpair (tk-dmrg/src/eigensolver/mod.rs:80-164):
// start vector ((i*7+13)%97)/97-0.5 when no guess is given, normalised;
// k = min(krylov_dim, dim) steps of the three-term recurrence with full
// re-orthogonalisation against every earlier Krylov vector; stop at a step
// whose beta < 1e-15; lowest eigenvalue of the tridiagonal matrix by 100
// steps of Sturm bisection (:179-233, :277-297).  Two defects of the
// reference are fixed, not copied: the Ritz vector is solved for by inverse
// iteration on the tridiagonal matrix (the reference's loop never solves and
// returns the normalised sum of Krylov vectors, :236-257), and the residual
// ||H x - E x|| is computed with an FP64 matvec (the reference reports 0).
//
// All vectors live on the device in the block layout.  The k-step recurrence
// is enqueued without host synchronisation (scalars stay in device memory)
// and captured once into a CUDA graph per (plan, k, precision); a Lanczos
// call then costs one graph launch plus the Ritz/residual epilogue.
//
// Split-precision plans follow each Lanczos run with up to `refine`
// Jacobi-Davidson steps in FP64 (one FP64 matvec each): Rayleigh-Ritz on an
// FP64 search space, whose new directions solve the projected correction
// equation (I-xx^T)(H-theta)(I-xx^T) t = -r by conjugate gradients with
// split-precision matvecs.  The energy and residual reported are those of
// FP64 matvecs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "tk_plan.cuh"

namespace tk {

struct LanczosGraph {
    int k = 0;
    int precision = -1;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~LanczosGraph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

void LanczosGraphDeleter::operator()(LanczosGraph* g) const { delete g; }

namespace {

constexpr int RT = 256;        // threads per reduction block
constexpr int RG = 2 * 152;    // reduction blocks (two per SM)
constexpr int MCH = 8;         // vectors per multidot pass

// partial[j*RG + b] = sum over this block's rows of V_j[i] * w[i], j < m.
__global__ void __launch_bounds__(RT) multidot_kernel(const double* __restrict__ V, int64_t ldv, int m,
                                                      const double* __restrict__ w, int64_t n,
                                                      double* __restrict__ partial) {
    const int j0 = blockIdx.y * MCH;
    const int mj = min(MCH, m - j0);
    double acc[MCH];
#pragma unroll
    for (int j = 0; j < MCH; ++j) acc[j] = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)RT + threadIdx.x; i < n; i += (int64_t)RG * RT) {
        const double wi = w[i];
#pragma unroll
        for (int j = 0; j < MCH; ++j)
            if (j < mj) acc[j] = fma(V[(int64_t)(j0 + j) * ldv + i], wi, acc[j]);
    }
    __shared__ double red[MCH][RT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < MCH; ++j) {
        double v = acc[j];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[j][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < mj) {
        double s = 0.0;
        for (int wv = 0; wv < RT / 32; ++wv) s += red[threadIdx.x][wv];
        partial[(int64_t)(j0 + threadIdx.x) * RG + blockIdx.x] = s;
    }
}

// out[j] = f(sum_b partial[j*RG+b]); mode 0: sum, 1: sqrt(sum).
__global__ void reduce_partial_kernel(const double* __restrict__ partial, double* __restrict__ out, int mode) {
    const int j = blockIdx.x;
    double s = 0.0;
    for (int b = threadIdx.x; b < RG; b += blockDim.x) s += partial[(int64_t)j * RG + b];
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int wv = 0; wv < (int)(blockDim.x / 32); ++wv) t += red[wv];
        out[j] = mode == 1 ? sqrt(fmax(t, 0.0)) : t;
    }
}

// w[i] -= sum_j c[j] V_j[i]
__global__ void gemv_sub_kernel(const double* __restrict__ V, int64_t ldv, int m, const double* __restrict__ c,
                                double* __restrict__ w, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double s = w[i];
        for (int j = 0; j < m; ++j) s = fma(-c[j], V[(int64_t)j * ldv + i], s);
        w[i] = s;
    }
}

// x[i] = sum_j z[j] V_j[i]
__global__ void gemv_kernel(const double* __restrict__ V, int64_t ldv, int m, const double* __restrict__ z,
                            double* __restrict__ x, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int j = 0; j < m; ++j) s = fma(z[j], V[(int64_t)j * ldv + i], s);
        x[i] = s;
    }
}

// w -= a*x + b*y with a, b read from device memory (b may be null).
__global__ void axpy2_kernel(double* __restrict__ w, const double* __restrict__ x, const double* pa,
                             const double* __restrict__ y, const double* pb, int64_t n) {
    const double a = *pa;
    const double b = pb ? *pb : 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double s = fma(-a, x[i], w[i]);
        if (pb) s = fma(-b, y[i], s);
        w[i] = s;
    }
}

// dst = src / *pnorm, or zeros when *pnorm < 1e-15 (breakdown); dst may be src.
__global__ void normalize_kernel(double* dst, const double* src, const double* pnorm,
                                 int64_t n) {
    const double nv = *pnorm;
    const double inv = nv < 1e-15 ? 0.0 : 1.0 / nv;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[i] * inv;
}

// y = a*x + b*y with host scalars
__global__ void axpby_kernel(double* __restrict__ y, const double* __restrict__ x, double a, double b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = fma(a, x[i], b * y[i]);
}

inline int vgrid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

struct Ws {
    double* V;      // k+1 vectors of length n
    double* w;      // work vector
    double* scal;   // alpha[0..K), beta[K..2K), c[2K..3K+1), misc
    double* part;   // RG * (K+1)
    double* vec;    // x / r / CG vectors: 4 * n
    int64_t n;
    int K;
};

inline double* ALPHA(const Ws& s) { return s.scal; }
inline double* BETA(const Ws& s) { return s.scal + s.K; }
inline double* COEF(const Ws& s) { return s.scal + 2 * s.K; }
inline double* MISC(const Ws& s) { return s.scal + 3 * s.K + 2; }

cudaError_t multidot(const Ws& ws, const double* V, int64_t ldv, int m, const double* w, double* out, int mode,
                     cudaStream_t s) {
    dim3 grid(RG, (m + MCH - 1) / MCH);
    multidot_kernel<<<grid, RT, 0, s>>>(V, ldv, m, w, ws.n, ws.part);
    reduce_partial_kernel<<<m, 128, 0, s>>>(ws.part, out, mode);
    return cudaGetLastError();
}

// Enqueues k Lanczos steps starting from the normalised V_0 already in place.
tk_status enqueue_steps(tk_heff2_plan* p, const Ws& ws, int k, int precision, cudaStream_t s) {
    const int64_t n = ws.n;
    for (int j = 0; j < k; ++j) {
        double* vj = ws.V + (int64_t)j * n;
        tk_status st = tk_heff2_apply_prec(p, vj, ws.w, s, precision);
        if (st != TK_OK) return st;
        cudaError_t e;
        if ((e = multidot(ws, vj, n, 1, ws.w, ALPHA(ws) + j, 0, s)) != cudaSuccess) return cuda_fail("multidot", e);
        axpy2_kernel<<<vgrid(n), 256, 0, s>>>(ws.w, vj, ALPHA(ws) + j, j > 0 ? ws.V + (int64_t)(j - 1) * n : nullptr,
                                               j > 0 ? BETA(ws) + (j - 1) : nullptr, n);
        // full re-orthogonalisation against V_0..V_j (blocked classical Gram-Schmidt)
        if ((e = multidot(ws, ws.V, n, j + 1, ws.w, COEF(ws), 0, s)) != cudaSuccess) return cuda_fail("multidot", e);
        gemv_sub_kernel<<<vgrid(n), 256, 0, s>>>(ws.V, n, j + 1, COEF(ws), ws.w, n);
        if ((e = multidot(ws, ws.w, n, 1, ws.w, BETA(ws) + j, 1, s)) != cudaSuccess) return cuda_fail("multidot", e);
        if (j + 1 < k) normalize_kernel<<<vgrid(n), 256, 0, s>>>(ws.V + (int64_t)(j + 1) * n, ws.w, BETA(ws) + j, n);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail("lanczos step", e);
    }
    return TK_OK;
}

// Sturm count (eigensolver/mod.rs:277-297).
int count_below(const std::vector<double>& d, const std::vector<double>& e, double mu) {
    int n = (int)d.size(), count = 0;
    double dp = d[0] - mu;
    if (dp < 0.0) ++count;
    for (int i = 1; i < n; ++i) {
        double q = (std::fabs(dp) < 1e-30) ? e[i - 1] * e[i - 1] / 1e-30 : e[i - 1] * e[i - 1] / dp;
        double dd = d[i] - mu - q;
        if (dd < 0.0) ++count;
        dp = dd;
    }
    return count;
}

// Lowest eigenvalue by bisection (eigensolver/mod.rs:210-233) and its
// eigenvector by inverse iteration with a tridiagonal LU solve.
double tridiag_lowest(const std::vector<double>& d, const std::vector<double>& e, std::vector<double>& z) {
    const int n = (int)d.size();
    double sum_e = 0.0;
    for (double x : e) sum_e += std::fabs(x);
    double lo = *std::min_element(d.begin(), d.end()) - sum_e;
    double hi = *std::max_element(d.begin(), d.end()) + sum_e;
    for (int it = 0; it < 100; ++it) {
        double mid = 0.5 * (lo + hi);
        if (count_below(d, e, mid) >= 1) hi = mid; else lo = mid;
    }
    const double lam = 0.5 * (lo + hi);
    z.assign(n, 1.0);
    if (n == 1) return lam;
    double scale = 0.0;
    for (int i = 0; i < n; ++i) scale = std::max(scale, std::fabs(d[i]));
    for (double x : e) scale = std::max(scale, std::fabs(x));
    const double shift = lam - 1e-13 * std::max(scale, 1.0);
    std::vector<double> cp(n), dp(n), b(n);
    for (int it = 0; it < 4; ++it) {
        // solve (T - shift I) y = z (Thomas algorithm with a tiny-pivot guard)
        double piv = d[0] - shift;
        if (std::fabs(piv) < 1e-300) piv = 1e-300;
        cp[0] = (n > 1) ? e[0] / piv : 0.0;
        dp[0] = z[0] / piv;
        for (int i = 1; i < n; ++i) {
            double den = d[i] - shift - e[i - 1] * cp[i - 1];
            if (std::fabs(den) < 1e-300) den = 1e-300;
            cp[i] = (i < n - 1) ? e[i] / den : 0.0;
            dp[i] = (z[i] - e[i - 1] * dp[i - 1]) / den;
        }
        b[n - 1] = dp[n - 1];
        for (int i = n - 2; i >= 0; --i) b[i] = dp[i] - cp[i] * b[i + 1];
        double nrm = 0.0;
        for (double x : b) nrm += x * x;
        nrm = std::sqrt(nrm);
        if (!(nrm > 0.0) || !std::isfinite(nrm)) break;
        for (int i = 0; i < n; ++i) z[i] = b[i] / nrm;
    }
    return lam;
}

tk_status read_scalar(const double* dev, double* host, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(host, dev, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? TK_OK : cuda_fail("read scalar", e);
}

// E = x.Hx, r = Hx - E x, returns ||r|| (FP64 matvec).  hx, r: work vectors.
tk_status fp64_residual(tk_heff2_plan* p, const Ws& ws, const double* x, double* hx, double* r, double* E,
                        double* rn, cudaStream_t s) {
    const int64_t n = ws.n;
    tk_status st = tk_heff2_apply_prec(p, x, hx, s, TK_PREC_FP64);
    if (st != TK_OK) return st;
    cudaError_t e;
    if ((e = multidot(ws, x, n, 1, hx, MISC(ws), 0, s)) != cudaSuccess) return cuda_fail("multidot", e);
    if ((st = read_scalar(MISC(ws), E, s)) != TK_OK) return st;
    if ((e = cudaMemcpyAsync(r, hx, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return cuda_fail("cudaMemcpyAsync", e);
    axpby_kernel<<<vgrid(n), 256, 0, s>>>(r, x, -*E, 1.0, n);
    if ((e = multidot(ws, r, n, 1, r, MISC(ws) + 1, 1, s)) != cudaSuccess) return cuda_fail("multidot", e);
    return read_scalar(MISC(ws) + 1, rn, s);
}

// ---- FP64 refinement of a split-precision eigenpair -------------------------
//
// Jacobi-Davidson with an FP64 search space: V holds up to RF_M orthonormal
// directions and HV their FP64 images (one FP64 matvec per direction).  Each
// outer step takes the Ritz pair (theta, x) of V^T H V, r = H x - theta x,
// then solves the correction equation (I-xx^T)(H - theta)(I-xx^T) t = -r
// approximately by `inner` conjugate-gradient steps whose matvecs run in the
// split precision, and adds t (orthogonalised against V) to V.  The split
// operator's error only slows the inner solve; theta and r always come from
// FP64 matvecs, so the residual falls to FP64 rounding level.

constexpr int RF_M = 8;         // refinement search-space size before a restart
constexpr int kInnerCg = 40;    // split-precision CG steps per refinement step, at most
constexpr int kCgCheck = 4;     // CG steps between convergence checks (one host read each)
constexpr double kCgRel = 1e-4; // CG stops once its residual fell by this factor

// CG scalars in device memory (rs):
//   rs[0] shift theta, rs[2] x.q, rs[3] p.q, rs[8 + (j&1)] rr of step j

__device__ __forceinline__ double cg_alpha(const double* rs, int j) {
    const double rr = rs[8 + (j & 1)], pq = rs[3];
    return (pq > 0.0 && rr > 0.0) ? rr / pq : 0.0;  // 0 freezes the iteration
}

// q -= theta p; partial[b] = x.q, partial[RG + b] = p.q over this block's rows
__global__ void __launch_bounds__(RT) cg_shift_dot2_kernel(double* __restrict__ q, const double* __restrict__ p,
                                                           const double* __restrict__ x, const double* rs, int64_t n,
                                                           double* __restrict__ partial) {
    const double th = rs[0];
    double a = 0.0, b = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)RT + threadIdx.x; i < n; i += (int64_t)RG * RT) {
        const double pi = p[i];
        const double qi = fma(-th, pi, q[i]);
        q[i] = qi;
        a = fma(x[i], qi, a);
        b = fma(pi, qi, b);
    }
    __shared__ double red[2][RT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
        red[0][warp] = a;
        red[1][warp] = b;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        double s = 0.0;
        for (int wv = 0; wv < RT / 32; ++wv) s += red[threadIdx.x][wv];
        partial[(int64_t)threadIdx.x * RG + blockIdx.x] = s;
    }
}

// q -= (x.q) x; t += alpha p; res -= alpha q; partial[b] = res.res
__global__ void __launch_bounds__(RT) cg_step_kernel(double* __restrict__ t, double* __restrict__ res,
                                                     const double* __restrict__ p, const double* __restrict__ q,
                                                     const double* __restrict__ x, const double* rs, int j, int64_t n,
                                                     double* __restrict__ partial) {
    const double alpha = cg_alpha(rs, j), xq = rs[2];
    double acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)RT + threadIdx.x; i < n; i += (int64_t)RG * RT) {
        double ri = res[i];
        if (alpha != 0.0) {
            t[i] = fma(alpha, p[i], t[i]);
            ri = fma(-alpha, fma(-xq, x[i], q[i]), ri);
            res[i] = ri;
        }
        acc = fma(ri, ri, acc);
    }
    __shared__ double red[RT / 32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int wv = 0; wv < RT / 32; ++wv) s += red[wv];
        partial[blockIdx.x] = s;
    }
}

// p = res + (rr_{j+1} / rr_j) p, unless step j was frozen
__global__ void cg_dir_kernel(double* __restrict__ p, const double* __restrict__ res, const double* rs, int j,
                              int64_t n) {
    if (cg_alpha(rs, j) == 0.0) return;
    const double beta = rs[8 + ((j + 1) & 1)] / rs[8 + (j & 1)];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = fma(beta, p[i], res[i]);
}

// Enqueues `iters` CG steps on (I-xx^T)(H_split - theta)(I-xx^T) t = -r with
// theta at rs[0]; t, res, p, q are work vectors.  No host synchronisation.
tk_status enqueue_correction(tk_heff2_plan* p, const Ws& ws, double* rs, const double* x, const double* r, double* t,
                             double* res, double* pv, double* q, int iters, int precision, cudaStream_t s, int* used) {
    const int64_t n = ws.n;
    cudaError_t e;
    *used = 0;
    if ((e = cudaMemsetAsync(t, 0, sizeof(double) * n, s)) != cudaSuccess) return cuda_fail("memset", e);
    if ((e = cudaMemsetAsync(res, 0, sizeof(double) * n, s)) != cudaSuccess) return cuda_fail("memset", e);
    axpby_kernel<<<vgrid(n), 256, 0, s>>>(res, r, -1.0, 0.0, n);
    if ((e = cudaMemcpyAsync(pv, res, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return cuda_fail("cudaMemcpyAsync", e);
    if ((e = multidot(ws, res, n, 1, res, rs + 8, 0, s)) != cudaSuccess) return cuda_fail("multidot", e);
    double rr0 = 0.0;
    tk_status st = read_scalar(rs + 8, &rr0, s);
    if (st != TK_OK) return st;
    for (int j = 0; j < iters; ++j) {
        if ((st = tk_heff2_apply_prec(p, pv, q, s, precision)) != TK_OK) return st;
        cg_shift_dot2_kernel<<<RG, RT, 0, s>>>(q, pv, x, rs, n, ws.part);
        reduce_partial_kernel<<<2, 128, 0, s>>>(ws.part, rs + 2, 0);
        cg_step_kernel<<<RG, RT, 0, s>>>(t, res, pv, q, x, rs, j, n, ws.part);
        reduce_partial_kernel<<<1, 128, 0, s>>>(ws.part, rs + 8 + ((j + 1) & 1), 0);
        cg_dir_kernel<<<vgrid(n), 256, 0, s>>>(pv, res, rs, j, n);
        *used = j + 1;
        // every kCgCheck steps: stop once the residual fell by kCgRel
        if ((j + 1) % kCgCheck == 0 && j + 1 < iters) {
            double rr = 0.0;
            if ((st = read_scalar(rs + 8 + ((j + 1) & 1), &rr, s)) != TK_OK) return st;
            if (!(rr > kCgRel * kCgRel * rr0)) break;
        }
    }
    e = cudaGetLastError();
    return e == cudaSuccess ? TK_OK : cuda_fail("correction solve", e);
}

// All eigenpairs of a symmetric m x m matrix (row-major, leading dim ld) by
// cyclic Jacobi rotations: w[i] and column i of z (row-major m x m).
void small_sym_eig(const std::vector<double>& g, int m, int ld, std::vector<double>& w, std::vector<double>& z) {
    std::vector<double> a((size_t)m * m);
    z.assign((size_t)m * m, 0.0);
    double frob = 0.0;
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) {
            a[(size_t)i * m + j] = g[(size_t)i * ld + j];
            frob += a[(size_t)i * m + j] * a[(size_t)i * m + j];
        }
    for (int i = 0; i < m; ++i) z[(size_t)i * m + i] = 1.0;
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = 0.0;
        for (int i = 0; i < m; ++i)
            for (int j = i + 1; j < m; ++j) off += a[(size_t)i * m + j] * a[(size_t)i * m + j];
        if (off <= 1e-34 * frob || off == 0.0) break;
        for (int pp = 0; pp < m; ++pp)
            for (int qq = pp + 1; qq < m; ++qq) {
                const double apq = a[(size_t)pp * m + qq];
                if (apq == 0.0) continue;
                const double th = (a[(size_t)qq * m + qq] - a[(size_t)pp * m + pp]) / (2.0 * apq);
                const double tn = (th >= 0.0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
                const double c = 1.0 / std::sqrt(tn * tn + 1.0), sn = tn * c;
                for (int k = 0; k < m; ++k) {  // A <- A P
                    const double akp = a[(size_t)k * m + pp], akq = a[(size_t)k * m + qq];
                    a[(size_t)k * m + pp] = c * akp - sn * akq;
                    a[(size_t)k * m + qq] = sn * akp + c * akq;
                }
                for (int k = 0; k < m; ++k) {  // A <- P^T A
                    const double apk = a[(size_t)pp * m + k], aqk = a[(size_t)qq * m + k];
                    a[(size_t)pp * m + k] = c * apk - sn * aqk;
                    a[(size_t)qq * m + k] = sn * apk + c * aqk;
                }
                for (int k = 0; k < m; ++k) {  // Z <- Z P
                    const double zkp = z[(size_t)k * m + pp], zkq = z[(size_t)k * m + qq];
                    z[(size_t)k * m + pp] = c * zkp - sn * zkq;
                    z[(size_t)k * m + qq] = sn * zkp + c * zkq;
                }
            }
    }
    w.resize(m);
    for (int i = 0; i < m; ++i) w[i] = a[(size_t)i * m + i];
}

// Lowest eigenpair (theta and the unit eigenvector) of a symmetric m x m
// matrix (row-major, leading dim ld): Householder reduction to tridiagonal
// form T = Q^T G Q, the lowest eigenvalue of T by Sturm bisection and its
// eigenvector by inverse iteration (tridiag_lowest, as the Lanczos solver
// does), then x = Q z.  About (4/3) m^3 flops, where cyclic Jacobi to full
// convergence spends some ten sweeps of 3 m^3 (for the search spaces of up to
// 60 directions this was most of a Davidson iteration's time on the host).
double small_sym_lowest(const std::vector<double>& g, int m, int ld, std::vector<double>& sv) {
    sv.assign(m, 0.0);
    if (m == 1) {
        sv[0] = 1.0;
        return g[0];
    }
    std::vector<double> a((size_t)m * m), q((size_t)m * m, 0.0), v(m), p(m), w(m);
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) a[(size_t)i * m + j] = g[(size_t)i * ld + j];
    for (int i = 0; i < m; ++i) q[(size_t)i * m + i] = 1.0;
    for (int k = 0; k + 2 < m; ++k) {
        // Householder vector v (zero above k + 1) mapping a[k+1.., k] onto e_{k+1}
        double sigma = 0.0;
        for (int i = k + 1; i < m; ++i) sigma += a[(size_t)i * m + k] * a[(size_t)i * m + k];
        if (sigma == 0.0) continue;
        const double x0 = a[(size_t)(k + 1) * m + k];
        const double alpha = x0 >= 0.0 ? -std::sqrt(sigma) : std::sqrt(sigma);
        for (int i = 0; i < m; ++i) v[i] = 0.0;
        v[k + 1] = x0 - alpha;
        for (int i = k + 2; i < m; ++i) v[i] = a[(size_t)i * m + k];
        const double vv = sigma - x0 * x0 + v[k + 1] * v[k + 1];
        if (vv == 0.0) continue;
        const double beta = 2.0 / vv;
        // A <- H A H with H = I - beta v v^T: p = beta A v, w = p - (beta / 2)(p.v) v,
        // A <- A - v w^T - w v^T (rows / columns k.. only)
        double pv = 0.0;
        for (int i = k; i < m; ++i) {
            double s2 = 0.0;
            for (int j = k + 1; j < m; ++j) s2 += a[(size_t)i * m + j] * v[j];
            p[i] = beta * s2;
            pv += p[i] * v[i];
        }
        for (int i = k; i < m; ++i) w[i] = p[i] - 0.5 * beta * pv * v[i];
        for (int i = k; i < m; ++i)
            for (int j = k; j < m; ++j) a[(size_t)i * m + j] -= v[i] * w[j] + w[i] * v[j];
        // Q <- Q H
        for (int i = 0; i < m; ++i) {
            double s2 = 0.0;
            for (int j = k + 1; j < m; ++j) s2 += q[(size_t)i * m + j] * v[j];
            s2 *= beta;
            for (int j = k + 1; j < m; ++j) q[(size_t)i * m + j] -= s2 * v[j];
        }
    }
    std::vector<double> d(m), e(m - 1), z;
    for (int i = 0; i < m; ++i) d[i] = a[(size_t)i * m + i];
    for (int i = 0; i + 1 < m; ++i) e[i] = a[(size_t)(i + 1) * m + i];
    const double lam = tridiag_lowest(d, e, z);
    double nrm = 0.0;
    for (int i = 0; i < m; ++i) {
        double s2 = 0.0;
        for (int j = 0; j < m; ++j) s2 += q[(size_t)i * m + j] * z[j];
        sv[i] = s2;
        nrm += s2 * s2;
    }
    nrm = std::sqrt(nrm);
    if (nrm > 0.0)
        for (double& x : sv) x /= nrm;
    // the Rayleigh quotient of the back-transformed vector (as accurate as the
    // bisection's bracket, and consistent with the vector used)
    double rq = 0.0;
    for (int i = 0; i < m; ++i) {
        double s2 = 0.0;
        for (int j = 0; j < m; ++j) s2 += g[(size_t)i * ld + j] * sv[j];
        rq += sv[i] * s2;
    }
    (void)lam;
    return rq;
}

// DavidsonSolver's diagonal preconditioner (eigensolver/mod.rs:427-437):
// t_i = r_i / (theta - d_i) where |theta - d_i| > 1e-14, else t_i = r_i.
__global__ void precondition_kernel(double* __restrict__ t, const double* __restrict__ r,
                                    const double* __restrict__ d, double theta, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double den = theta - d[i];
        t[i] = fabs(den) > 1e-14 ? r[i] / den : r[i];
    }
}

// Search space of the FP64 subspace solver: V (orthonormal directions), HV
// (their FP64 images), host-visible scalars sc and reduction partials.
struct Subspace {
    double* V;
    double* HV;
    double* sc;  // [0, M) coefficients, [M] a norm, [M+8, M+24) CG scalars
    int M;
    int matvecs = 0, fp64_matvecs = 0;
};

struct SubspaceCfg {
    int max_iter;
    double tol;
    const double* diag;   // Davidson preconditioner (device, block layout) or null
    int inner;            // > 0: correction by `inner` CG steps in `inner_prec`
    int inner_prec;
    bool restart_matvec;  // restart as DavidsonSolver: recompute H y, drop the correction
    bool have_hx;         // hx = H x on entry (no first matvec)
};

// Davidson / Jacobi-Davidson on an FP64 search space (DavidsonSolver::
// lowest_eigenpair, eigensolver/mod.rs:325-517):
//   Rayleigh-Ritz on V^T H V (its upper triangle is V_i . HV_j, :368-376),
//   y = V c, r = HV c - theta y (:389-411), stop when |r| < tol (:413-422);
//   the correction is r (optionally diagonal-preconditioned) or, with
//   inner > 0, an approximate solution of the projected correction equation;
//   it is orthogonalised against V, falls back to the orthogonalised raw
//   residual when it collapses below 1e-14 (:449-477), and is added with one
//   FP64 matvec; at M directions the space restarts from y (:485-500).
// Orthogonalisation is two passes of blocked classical Gram-Schmidt (the
// reference uses one modified Gram-Schmidt pass), and the small eigenproblem
// uses cyclic Jacobi with a relative stopping rule.
// On exit x (unit), hx, r = hx - E x and rn describe the last Ritz pair.
tk_status subspace_solve(tk_heff2_plan* p, const Ws& ws, Subspace& sp, const SubspaceCfg& cfg, double* x, double* hx,
                         double* r, double* E, double* rn, bool* converged, cudaStream_t s) {
    const int64_t n = ws.n;
    const int M = sp.M;
    double* t = ws.vec + 2 * n;
    double* sc = sp.sc;
    double* rs = sp.sc + M + 8;
    cudaError_t e;
    tk_status st;
    std::vector<double> G((size_t)M * M, 0.0), col(M + 1), cvec;
    *converged = false;
    // V_0 = x / |x|, HV_0 = H V_0
    if ((e = multidot(ws, x, n, 1, x, sc + M, 1, s)) != cudaSuccess) return cuda_fail("multidot", e);
    normalize_kernel<<<vgrid(n), 256, 0, s>>>(sp.V, x, sc + M, n);
    if (cfg.have_hx) {
        normalize_kernel<<<vgrid(n), 256, 0, s>>>(sp.HV, hx, sc + M, n);
    } else {
        if ((st = tk_heff2_apply_prec(p, sp.V, sp.HV, s, TK_PREC_FP64)) != TK_OK) return st;
        ++sp.matvecs;
        ++sp.fp64_matvecs;
    }
    auto add_column = [&](int j) -> tk_status {  // G[i][j] = G[j][i] = V_i . HV_j, i <= j
        cudaError_t e2 = multidot(ws, sp.V, n, j + 1, sp.HV + (int64_t)j * n, sc, 0, s);
        if (e2 != cudaSuccess) return cuda_fail("multidot", e2);
        if ((e2 = cudaMemcpyAsync(col.data(), sc, sizeof(double) * (j + 1), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return cuda_fail("cudaMemcpyAsync", e2);
        if ((e2 = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail("subspace step", e2);
        for (int i = 0; i <= j; ++i) G[(size_t)i * M + j] = G[(size_t)j * M + i] = col[i];
        return TK_OK;
    };
    if ((st = add_column(0)) != TK_OK) return st;
    int m = 1;
    double theta = G[0];
    for (int it = 0; it < cfg.max_iter; ++it) {
        if (plan_cancelled(p, s, "davidson")) return TK_ERR_CANCELLED;
        // Ritz pair and residual
        theta = small_sym_lowest(G, m, M, cvec);
        if ((e = cudaMemcpyAsync(sc, cvec.data(), sizeof(double) * m, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return cuda_fail("cudaMemcpyAsync", e);
        gemv_kernel<<<vgrid(n), 256, 0, s>>>(sp.V, n, m, sc, x, n);
        gemv_kernel<<<vgrid(n), 256, 0, s>>>(sp.HV, n, m, sc, hx, n);
        if ((e = cudaMemcpyAsync(r, hx, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
            return cuda_fail("cudaMemcpyAsync", e);
        axpby_kernel<<<vgrid(n), 256, 0, s>>>(r, x, -theta, 1.0, n);
        if ((e = multidot(ws, r, n, 1, r, sc + M, 1, s)) != cudaSuccess) return cuda_fail("multidot", e);
        if ((st = read_scalar(sc + M, rn, s)) != TK_OK) return st;
        *E = theta;
        if (*rn < cfg.tol) {
            *converged = true;
            break;
        }
        // correction
        if (cfg.inner > 0) {
            if ((e = cudaMemcpyAsync(rs, &theta, sizeof(double), cudaMemcpyHostToDevice, s)) != cudaSuccess)
                return cuda_fail("cudaMemcpyAsync", e);
            int used = 0;
            if ((st = enqueue_correction(p, ws, rs, x, r, t, ws.V, ws.V + n, ws.V + 2 * n, cfg.inner, cfg.inner_prec,
                                         s, &used)) != TK_OK)
                return st;
            sp.matvecs += used;
        } else if (cfg.diag) {
            precondition_kernel<<<vgrid(n), 256, 0, s>>>(t, r, cfg.diag, theta, n);
        } else if ((e = cudaMemcpyAsync(t, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) {
            return cuda_fail("cudaMemcpyAsync", e);
        }
        double cnorm = 0.0;
        for (int attempt = 0; attempt < 2; ++attempt) {
            for (int pass = 0; pass < 2; ++pass) {
                if ((e = multidot(ws, sp.V, n, m, t, sc, 0, s)) != cudaSuccess) return cuda_fail("multidot", e);
                gemv_sub_kernel<<<vgrid(n), 256, 0, s>>>(sp.V, n, m, sc, t, n);
            }
            if ((e = multidot(ws, t, n, 1, t, sc + M, 1, s)) != cudaSuccess) return cuda_fail("multidot", e);
            if ((st = read_scalar(sc + M, &cnorm, s)) != TK_OK) return st;
            if (cnorm >= 1e-14 || attempt == 1) break;
            // the correction collapsed into span(V): use the raw residual
            if ((e = cudaMemcpyAsync(t, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
                return cuda_fail("cudaMemcpyAsync", e);
        }
        if (cnorm < 1e-14) break;  // converged or stagnated
        if (m >= M) {
            if (m >= n) break;  // the space is complete
            if ((e = cudaMemcpyAsync(sp.V, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
                return cuda_fail("cudaMemcpyAsync", e);
            if (cfg.restart_matvec) {
                if ((st = tk_heff2_apply_prec(p, sp.V, sp.HV, s, TK_PREC_FP64)) != TK_OK) return st;
                ++sp.matvecs;
                ++sp.fp64_matvecs;
                m = 1;
                if ((st = add_column(0)) != TK_OK) return st;
                continue;
            }
            if ((e = cudaMemcpyAsync(sp.HV, hx, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
                return cuda_fail("cudaMemcpyAsync", e);
            G[0] = theta;
            m = 1;
            // t is orthogonal to the old span, which contains y: append it below
        }
        double* vm = sp.V + (int64_t)m * n;
        normalize_kernel<<<vgrid(n), 256, 0, s>>>(vm, t, sc + M, n);
        if ((st = tk_heff2_apply_prec(p, vm, sp.HV + (int64_t)m * n, s, TK_PREC_FP64)) != TK_OK) return st;
        ++sp.matvecs;
        ++sp.fp64_matvecs;
        if ((st = add_column(m)) != TK_OK) return st;
        ++m;
    }
    e = cudaGetLastError();
    return e == cudaSuccess ? TK_OK : cuda_fail("subspace solve", e);
}

// Lanczos workspace for k steps (allocated on first use, grown on demand).
tk_status ensure_lanczos_ws(tk_heff2_plan* p, int k, int64_t n, Ws* ws) {
    cudaError_t e;
    if (p->lz_cap_k < k) {
        p->lz_basis.reset();
        p->lz_w.reset();
        p->lz_scal.reset();
        p->lz_part.reset();
        p->lz_vec.reset();
        p->lz_graph.reset();
        const int kk = std::max(k, 2);
        if ((e = p->lz_basis.alloc((size_t)(kk + 1) * n)) != cudaSuccess) return cuda_fail("alloc basis", e);
        if ((e = p->lz_w.alloc((size_t)n)) != cudaSuccess) return cuda_fail("alloc w", e);
        if ((e = p->lz_scal.alloc((size_t)(4 * kk + 16))) != cudaSuccess) return cuda_fail("alloc scal", e);
        if ((e = p->lz_part.alloc((size_t)RG * (kk + 1))) != cudaSuccess) return cuda_fail("alloc part", e);
        if ((e = p->lz_vec.alloc((size_t)4 * n)) != cudaSuccess) return cuda_fail("alloc vec", e);
        p->lz_cap_k = k;
    }
    *ws = Ws{p->lz_basis.p, p->lz_w.p, p->lz_scal.p, p->lz_part.p, p->lz_vec.p, n, std::max(p->lz_cap_k, 2)};
    return TK_OK;
}

// Search space of M directions; `ws` gets a partials buffer for M-wide multidots.
tk_status ensure_subspace(tk_heff2_plan* p, int M, int64_t n, Ws* ws, Subspace* sp) {
    cudaError_t e;
    if (p->sub_cap < M) {
        p->sub_cap = 0;
        if ((e = p->sub_v.alloc((size_t)M * n)) != cudaSuccess) return cuda_fail("alloc search space", e);
        if ((e = p->sub_hv.alloc((size_t)M * n)) != cudaSuccess) return cuda_fail("alloc search space", e);
        if ((e = p->sub_sc.alloc((size_t)M + 32)) != cudaSuccess) return cuda_fail("alloc search space", e);
        if ((e = p->sub_part.alloc((size_t)RG * (M + 1))) != cudaSuccess) return cuda_fail("alloc search space", e);
        p->sub_cap = M;
    }
    ws->part = p->sub_part.p;
    *sp = Subspace{p->sub_v.p, p->sub_hv.p, p->sub_sc.p, M};
    return TK_OK;
}

struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev) {
        cudaGetDevice(&prev);
        cudaSetDevice(dev);
    }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

// out = X1 + i X2 in the vector's own complex form: with nc = 2 the length-2n
// vectors hold (re; im) halves and multiplication by i maps (x; y) to (-y; x).
__global__ void expm_assemble_kernel(double* __restrict__ out_re, double* __restrict__ out_im,
                                     const double* __restrict__ x1, const double* __restrict__ x2, int64_t n, int nc) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (nc == 2) {
            out_re[i] = x1[i] - x2[n + i];
            if (out_im) out_im[i] = x1[n + i] + x2[i];
        } else {
            out_re[i] = x1[i];
            if (out_im) out_im[i] = x2[i];
        }
    }
}

// exp(alpha H) v for the plan's H and a real or complex v: Lanczos with full
// re-orthogonalisation on the real vector v~ = v (nc = 1) or (Re v; Im v)
// (nc = 2; a real H acts on each half, a complex Hermitian H as the real
// symmetric [[Re H, -Im H], [Im H, Re H]]), whose recurrence coefficients are
// those of the complex Lanczos process; exp(alpha T_m) e_1
// from the eigendecomposition of the tridiagonal T_m (any complex alpha);
// result = sum_k c_k V_k with complex c_k.
tk_status expm_run(tk_heff2_plan* p, const Ws& ws, int nc, int64_t n, int m, double tol, double are, double aim,
                   const double* vre, const double* vim, double* ore, double* oim, double* x2, tk_expm_result* res,
                   cudaStream_t s) {
    const int64_t nn = ws.n;  // nc * n
    cudaError_t e;
    tk_status st;
    if ((e = cudaMemcpyAsync(ws.V, vre, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return cuda_fail("cudaMemcpyAsync", e);
    if (nc == 2) {
        e = vim ? cudaMemcpyAsync(ws.V + n, vim, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)
                : cudaMemsetAsync(ws.V + n, 0, sizeof(double) * n, s);
        if (e != cudaSuccess) return cuda_fail("cudaMemcpyAsync", e);
    }
    if ((e = multidot(ws, ws.V, nn, 1, ws.V, MISC(ws), 1, s)) != cudaSuccess) return cuda_fail("multidot", e);
    double beta0 = 0.0;
    if ((st = read_scalar(MISC(ws), &beta0, s)) != TK_OK) return st;
    res->input_norm = beta0;
    if (beta0 < 1e-30) {  // exp_krylov_f64 returns zeros (tdvp/mod.rs:214-217)
        if ((e = cudaMemsetAsync(ore, 0, sizeof(double) * n, s)) != cudaSuccess) return cuda_fail("memset", e);
        if (oim && (e = cudaMemsetAsync(oim, 0, sizeof(double) * n, s)) != cudaSuccess) return cuda_fail("memset", e);
        return TK_OK;
    }
    normalize_kernel<<<vgrid(nn), 256, 0, s>>>(ws.V, ws.V, MISC(ws), nn);
    for (int j = 0; j < m; ++j) {
        if (j % 8 == 0 && plan_cancelled(p, s, "krylov exponential")) return TK_ERR_CANCELLED;
        double* vj = ws.V + (int64_t)j * nn;
        if (p->is_complex) {  // complex Hermitian H on (re; im): one complex matvec
            if ((st = tk_heff2_apply_complex_s(p, vj, vj + n, ws.w, ws.w + n, s)) != TK_OK) return st;
            res->matvec_count += 1;
        } else {  // real H: each half on its own
            for (int h = 0; h < nc; ++h)
                if ((st = tk_heff2_apply_prec(p, vj + h * n, ws.w + h * n, s, p->precision)) != TK_OK) return st;
            res->matvec_count += nc;
        }
        if ((e = multidot(ws, vj, nn, 1, ws.w, ALPHA(ws) + j, 0, s)) != cudaSuccess) return cuda_fail("multidot", e);
        axpy2_kernel<<<vgrid(nn), 256, 0, s>>>(ws.w, vj, ALPHA(ws) + j, j > 0 ? ws.V + (int64_t)(j - 1) * nn : nullptr,
                                                j > 0 ? BETA(ws) + (j - 1) : nullptr, nn);
        for (int pass = 0; pass < 2; ++pass) {
            if ((e = multidot(ws, ws.V, nn, j + 1, ws.w, COEF(ws), 0, s)) != cudaSuccess) return cuda_fail("multidot", e);
            gemv_sub_kernel<<<vgrid(nn), 256, 0, s>>>(ws.V, nn, j + 1, COEF(ws), ws.w, nn);
        }
        if ((e = multidot(ws, ws.w, nn, 1, ws.w, BETA(ws) + j, 1, s)) != cudaSuccess) return cuda_fail("multidot", e);
        if (j + 1 < m) normalize_kernel<<<vgrid(nn), 256, 0, s>>>(ws.V + (int64_t)(j + 1) * nn, ws.w, BETA(ws) + j, nn);
    }
    std::vector<double> ab(2 * (size_t)ws.K);
    if ((e = cudaMemcpyAsync(ab.data(), ws.scal, sizeof(double) * 2 * ws.K, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_fail("cudaMemcpyAsync", e);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail("krylov exponential", e);
    // happy breakdown (tdvp/mod.rs:250-254): the space is invariant after step j
    int am = m;
    for (int j = 0; j < m; ++j)
        if (ab[ws.K + j] < tol) {
            am = j + 1;
            break;
        }
    res->krylov_used = am;
    std::vector<double> T((size_t)am * am, 0.0), w, z;
    for (int j = 0; j < am; ++j) {
        T[(size_t)j * am + j] = ab[j];
        if (j + 1 < am) T[(size_t)j * am + j + 1] = T[(size_t)(j + 1) * am + j] = ab[ws.K + j];
    }
    small_sym_eig(T, am, am, w, z);
    // c_k = beta0 * sum_l z[k][l] exp(alpha w_l) z[0][l]
    std::vector<double> c(2 * (size_t)am, 0.0);
    for (int l = 0; l < am; ++l) {
        const double mag = std::exp(are * w[l]), ph = aim * w[l];
        const double er = mag * std::cos(ph), ei = mag * std::sin(ph);
        for (int k = 0; k < am; ++k) {
            const double f = beta0 * z[(size_t)k * am + l] * z[l];
            c[k] += f * er;
            c[am + k] += f * ei;
        }
    }
    if ((e = cudaMemcpyAsync(COEF(ws), c.data(), sizeof(double) * 2 * am, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail("cudaMemcpyAsync", e);
    gemv_kernel<<<vgrid(nn), 256, 0, s>>>(ws.V, nn, am, COEF(ws), ws.w, nn);
    gemv_kernel<<<vgrid(nn), 256, 0, s>>>(ws.V, nn, am, COEF(ws) + am, x2, nn);
    expm_assemble_kernel<<<vgrid(n), 256, 0, s>>>(ore, oim, ws.w, x2, n, nc);
    e = cudaGetLastError();
    return e == cudaSuccess ? TK_OK : cuda_fail("krylov exponential", e);
}

}  // namespace
}  // namespace tk

using namespace tk;

extern "C" tk_status tk_expm_krylov(tk_heff2_plan* p, const tk_expm_cfg* cfg, double alpha_re, double alpha_im,
                                    const double* v_re, const double* v_im, double* out_re, double* out_im,
                                    tk_expm_result* res, void* stream) {
    if (!p || !cfg || !res || !v_re || !out_re) {
        set_error("tk_expm_krylov: null argument");
        return TK_ERR_INVALID_ARG;
    }
    *res = tk_expm_result{};
    const bool cplx = v_im != nullptr || p->is_complex;
    if (!out_im && (cplx || alpha_im != 0.0)) {
        set_error("tk_expm_krylov: a complex result needs out_im");
        return TK_ERR_INVALID_ARG;
    }
    if (cfg->krylov_dim < 1 || cfg->krylov_dim > 256 || !(cfg->tol >= 0.0)) {
        set_error("tk_expm_krylov: krylov_dim must be in [1, 256] and tol >= 0");
        return TK_ERR_INVALID_ARG;
    }
    const int64_t n = p->host.total;
    if (n == 0) {
        set_error("tk_expm_krylov: empty two-site space");
        return TK_ERR_INVALID_ARG;
    }
    DeviceScope scope(p->device);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e;
    const int nc = cplx ? 2 : 1;
    const int m = (int)std::min<int64_t>(cfg->krylov_dim, nc * n);  // min(krylov_dim, dim) (tdvp/mod.rs:207)
    const int64_t nn = nc * n;
    if (p->ex_cap_m < m || p->ex_cap_n < nn) {
        const int mm = std::max(m, p->ex_cap_m);
        const int64_t nmax = std::max(nn, p->ex_cap_n);
        p->ex_cap_m = 0;
        if ((e = p->ex_basis.alloc((size_t)(mm + 1) * nmax)) != cudaSuccess) return cuda_fail("alloc krylov basis", e);
        if ((e = p->ex_w.alloc((size_t)nmax)) != cudaSuccess) return cuda_fail("alloc krylov", e);
        if ((e = p->ex_x2.alloc((size_t)nmax)) != cudaSuccess) return cuda_fail("alloc krylov", e);
        if ((e = p->ex_scal.alloc((size_t)(4 * (mm + 2) + 16))) != cudaSuccess) return cuda_fail("alloc krylov", e);
        if ((e = p->ex_part.alloc((size_t)RG * (mm + 1))) != cudaSuccess) return cuda_fail("alloc krylov", e);
        p->ex_cap_m = mm;
        p->ex_cap_n = nmax;
    }
    Ws ws{p->ex_basis.p, p->ex_w.p, p->ex_scal.p, p->ex_part.p, nullptr, nn, std::max(p->ex_cap_m, 2)};
    tk_status st = expm_run(p, ws, nc, n, m, cfg->tol, alpha_re, alpha_im, v_re, v_im, out_re, out_im, p->ex_x2.p,
                            res, s);
    if (st != TK_OK) return st;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail("krylov exponential", e);
    if (p->tc && (st = tc_check_error(*p->tc, s)) != TK_OK) return st;
    return TK_OK;
}

extern "C" tk_status tk_lanczos_lowest(tk_heff2_plan* p, const tk_lanczos_cfg* cfg, const double* x0_dev,
                                       double* evec_dev, tk_eigen_result* out, void* stream) {
    if (!p || !cfg || !out || !evec_dev) {
        set_error("tk_lanczos_lowest: null argument");
        return TK_ERR_INVALID_ARG;
    }
    *out = tk_eigen_result{};
    const int64_t n = p->host.total;
    if (n == 0) {
        set_error("tk_lanczos_lowest: empty two-site space");
        return TK_ERR_INVALID_ARG;
    }
    if (cfg->krylov_dim < 1 || cfg->krylov_dim > 512 || cfg->max_restarts < 0 || cfg->refine < 0) {
        set_error("tk_lanczos_lowest: krylov_dim must be in [1, 512], restarts and refine >= 0");
        return TK_ERR_INVALID_ARG;
    }
    DeviceScope scope(p->device);
    const int k = (int)std::min<int64_t>(cfg->krylov_dim, n);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e;
    Ws ws;
    tk_status st = ensure_lanczos_ws(p, k, n, &ws);
    if (st != TK_OK) return st;
    double* x = evec_dev;
    double* hx = ws.vec;
    double* r = ws.vec + n;
    const int lz_prec = p->precision;
    // start vector -> x
    if (x0_dev) {
        if (x0_dev != x && (e = cudaMemcpyAsync(x, x0_dev, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
            return cuda_fail("cudaMemcpyAsync", e);
    } else if ((e = launch_fill_start_vector(x, n, s)) != cudaSuccess) {
        return cuda_fail("start vector", e);
    }
    int matvecs = 0, fp64_matvecs = 0, restarts = 0;
    double E = 0.0, rn = INFINITY;
    for (;;) {
        if (plan_cancelled(p, s, "lanczos")) return TK_ERR_CANCELLED;
        // V_0 = x / |x|
        if ((e = multidot(ws, x, n, 1, x, MISC(ws) + 4, 1, s)) != cudaSuccess) return cuda_fail("multidot", e);
        normalize_kernel<<<vgrid(n), 256, 0, s>>>(ws.V, x, MISC(ws) + 4, n);
        // k steps, through a cached CUDA graph
        LanczosGraph* g = p->lz_graph.get();
        if (!g || g->k != k || g->precision != lz_prec) {
            p->lz_graph.reset(new LanczosGraph);
            g = p->lz_graph.get();
            g->k = k;
            g->precision = lz_prec;
            cudaStream_t cs = p->stream;
            if ((e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
                return cuda_fail("cudaStreamBeginCapture", e);
            st = enqueue_steps(p, ws, k, lz_prec, cs);
            cudaGraph_t graph = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
            if (st != TK_OK) {
                if (graph) cudaGraphDestroy(graph);
                p->lz_graph.reset();
                return st;
            }
            if (e2 != cudaSuccess) {
                p->lz_graph.reset();
                return cuda_fail("cudaStreamEndCapture", e2);
            }
            g->graph = graph;
            if ((e = cudaGraphInstantiate(&g->exec, graph, 0)) != cudaSuccess) {
                p->lz_graph.reset();
                return cuda_fail("cudaGraphInstantiate", e);
            }
        }
        if ((e = cudaGraphLaunch(g->exec, s)) != cudaSuccess) return cuda_fail("cudaGraphLaunch", e);
        matvecs += k;
        if (lz_prec == TK_PREC_FP64) fp64_matvecs += k;
        // tridiagonal coefficients to the host
        std::vector<double> hs(2 * (size_t)ws.K);
        if ((e = cudaMemcpyAsync(hs.data(), ws.scal, sizeof(double) * 2 * ws.K, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return cuda_fail("cudaMemcpyAsync", e);
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail("lanczos run", e);
        int m = k;
        for (int j = 0; j < k; ++j)
            if (hs[ws.K + j] < 1e-15) {
                m = j + 1;
                break;
            }
        std::vector<double> d(hs.begin(), hs.begin() + m), off(hs.begin() + ws.K, hs.begin() + ws.K + (m - 1));
        std::vector<double> z;
        tridiag_lowest(d, off, z);
        // Ritz vector x = V z, normalised
        if ((e = cudaMemcpyAsync(COEF(ws), z.data(), sizeof(double) * m, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return cuda_fail("cudaMemcpyAsync", e);
        gemv_kernel<<<vgrid(n), 256, 0, s>>>(ws.V, n, m, COEF(ws), x, n);
        if ((e = multidot(ws, x, n, 1, x, MISC(ws) + 5, 1, s)) != cudaSuccess) return cuda_fail("multidot", e);
        normalize_kernel<<<vgrid(n), 256, 0, s>>>(x, x, MISC(ws) + 5, n);
        // FP64 energy and residual
        if ((st = fp64_residual(p, ws, x, hx, r, &E, &rn, s)) != TK_OK) return st;
        ++fp64_matvecs;
        ++matvecs;
        // split precision: FP64 Jacobi-Davidson refinement
        if (lz_prec != TK_PREC_FP64 && cfg->refine > 0 && rn > cfg->tol) {
            Ws ws2 = ws;
            Subspace sp;
            if ((st = ensure_subspace(p, RF_M, n, &ws2, &sp)) != TK_OK) return st;
            SubspaceCfg sc{cfg->refine, cfg->tol, nullptr, kInnerCg, lz_prec, false, true};
            bool conv = false;
            if ((st = subspace_solve(p, ws2, sp, sc, x, hx, r, &E, &rn, &conv, s)) != TK_OK) return st;
            matvecs += sp.matvecs;
            fp64_matvecs += sp.fp64_matvecs;
        }
        if (rn <= cfg->tol || restarts >= cfg->max_restarts) break;
        ++restarts;
    }
    if (p->tc && (st = tc_check_error(*p->tc, s)) != TK_OK) return st;
    out->eigenvalue = E;
    out->residual_norm = rn;
    out->converged = rn <= cfg->tol ? 1 : 0;
    out->matvec_count = matvecs;
    out->fp64_matvec_count = fp64_matvecs;
    out->restarts = restarts;
    return TK_OK;
}

extern "C" tk_status tk_davidson_lowest(tk_heff2_plan* p, const tk_davidson_cfg* cfg, const double* x0_dev,
                                        double* evec_dev, tk_eigen_result* out, void* stream) {
    if (!p || !cfg || !out || !evec_dev) {
        set_error("tk_davidson_lowest: null argument");
        return TK_ERR_INVALID_ARG;
    }
    *out = tk_eigen_result{};
    const int64_t n = p->host.total;
    if (n == 0) {
        set_error("tk_davidson_lowest: empty two-site space");
        return TK_ERR_INVALID_ARG;
    }
    if (cfg->max_subspace < 1 || cfg->max_subspace > 256 || cfg->max_iter < 0 || cfg->inner < 0 ||
        cfg->inner > 1000) {
        set_error("tk_davidson_lowest: max_subspace must be in [1, 256], max_iter >= 0, inner in [0, 1000]");
        return TK_ERR_INVALID_ARG;
    }
    DeviceScope scope(p->device);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e;
    Ws ws;
    tk_status st = ensure_lanczos_ws(p, 2, n, &ws);
    if (st != TK_OK) return st;
    const int M = (int)std::min<int64_t>(cfg->max_subspace, n);
    Subspace sp;
    if ((st = ensure_subspace(p, M, n, &ws, &sp)) != TK_OK) return st;
    double* x = evec_dev;
    if (x0_dev) {
        if (x0_dev != x && (e = cudaMemcpyAsync(x, x0_dev, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
            return cuda_fail("cudaMemcpyAsync", e);
    } else if ((e = launch_fill_start_vector(x, n, s)) != cudaSuccess) {
        return cuda_fail("start vector", e);
    }
    const int inner = p->precision != TK_PREC_FP64 ? cfg->inner : 0;
    SubspaceCfg sc{cfg->max_iter, cfg->tol, cfg->diagonal, inner, p->precision, true, false};
    double E = 0.0, rn = INFINITY;
    bool conv = false;
    if ((st = subspace_solve(p, ws, sp, sc, x, ws.vec, ws.vec + n, &E, &rn, &conv, s)) != TK_OK) return st;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail("davidson", e);
    if (p->tc && (st = tc_check_error(*p->tc, s)) != TK_OK) return st;
    out->eigenvalue = E;
    out->residual_norm = rn;
    out->converged = conv ? 1 : 0;
    out->matvec_count = sp.matvecs;
    out->fp64_matvec_count = sp.fp64_matvecs;
    out->restarts = 0;
    return TK_OK;
}
