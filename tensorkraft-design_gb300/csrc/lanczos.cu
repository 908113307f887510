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
// Split-precision plans add `refine` FP64 correction steps after the
// Lanczos run: r = H x - E x with an FP64 matvec, then the projected
// correction equation (I-xx^T)(H-E)(I-xx^T) t = -r solved by conjugate
// gradients with split-precision matvecs, x <- (x+t)/|x+t|.  The energy and
// residual reported are those of FP64 matvecs.
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

// dst = src / *pnorm, or zeros when *pnorm < 1e-15 (breakdown).
__global__ void normalize_kernel(double* __restrict__ dst, const double* __restrict__ src, const double* pnorm,
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

tk_status dot_host(const Ws& ws, const double* a, const double* b, double* out, cudaStream_t s) {
    cudaError_t e = multidot(ws, a, ws.n, 1, b, MISC(ws) + 2, 0, s);
    if (e != cudaSuccess) return cuda_fail("multidot", e);
    return read_scalar(MISC(ws) + 2, out, s);
}

// One correction step: CG on (I-xx^T)(H_lp - E)(I-xx^T) t = -r.
tk_status correction_step(tk_heff2_plan* p, const Ws& ws, double* x, const double* r, double E, int iters,
                          int precision, cudaStream_t s) {
    const int64_t n = ws.n;
    double* t = ws.vec + 2 * n;
    double* res = ws.vec + 3 * n;
    double* pv = ws.V;          // reuse the Krylov storage as CG work space
    double* q = ws.V + n;
    cudaError_t e;
    if ((e = cudaMemsetAsync(t, 0, sizeof(double) * n, s)) != cudaSuccess) return cuda_fail("memset", e);
    // res = -r ; p = res
    if ((e = cudaMemsetAsync(res, 0, sizeof(double) * n, s)) != cudaSuccess) return cuda_fail("memset", e);
    axpby_kernel<<<vgrid(n), 256, 0, s>>>(res, r, -1.0, 0.0, n);
    if ((e = cudaMemcpyAsync(pv, res, sizeof(double) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return cuda_fail("cudaMemcpyAsync", e);
    double rr = 0.0;
    tk_status st = dot_host(ws, res, res, &rr, s);
    if (st != TK_OK) return st;
    const double rr0 = rr;
    for (int it = 0; it < iters && rr > 1e-24 * rr0 && rr > 0.0; ++it) {
        if ((st = tk_heff2_apply_prec(p, pv, q, s, precision)) != TK_OK) return st;
        axpby_kernel<<<vgrid(n), 256, 0, s>>>(q, pv, -E, 1.0, n);
        double xq = 0.0;
        if ((st = dot_host(ws, x, q, &xq, s)) != TK_OK) return st;
        axpby_kernel<<<vgrid(n), 256, 0, s>>>(q, x, -xq, 1.0, n);
        double pq = 0.0;
        if ((st = dot_host(ws, pv, q, &pq, s)) != TK_OK) return st;
        if (!(pq > 0.0)) break;  // operator not positive on this direction: stop
        const double alpha = rr / pq;
        axpby_kernel<<<vgrid(n), 256, 0, s>>>(t, pv, alpha, 1.0, n);
        axpby_kernel<<<vgrid(n), 256, 0, s>>>(res, q, -alpha, 1.0, n);
        double rr_new = 0.0;
        if ((st = dot_host(ws, res, res, &rr_new, s)) != TK_OK) return st;
        const double beta = rr_new / rr;
        axpby_kernel<<<vgrid(n), 256, 0, s>>>(pv, res, 1.0, beta, n);
        rr = rr_new;
    }
    // x <- (x + t) / |x + t|
    axpby_kernel<<<vgrid(n), 256, 0, s>>>(x, t, 1.0, 1.0, n);
    if ((e = multidot(ws, x, n, 1, x, MISC(ws) + 3, 1, s)) != cudaSuccess) return cuda_fail("multidot", e);
    normalize_kernel<<<vgrid(n), 256, 0, s>>>(x, x, MISC(ws) + 3, n);
    e = cudaGetLastError();
    return e == cudaSuccess ? TK_OK : cuda_fail("correction step", e);
}

}  // namespace
}  // namespace tk

using namespace tk;

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
    int prev_dev = -1;
    cudaGetDevice(&prev_dev);
    cudaSetDevice(p->device);
    struct Restore {
        int d;
        ~Restore() {
            if (d >= 0) cudaSetDevice(d);
        }
    } restore{prev_dev};
    const int k = (int)std::min<int64_t>(cfg->krylov_dim, n);
    cudaStream_t s = (cudaStream_t)stream;
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
    Ws ws{p->lz_basis.p, p->lz_w.p, p->lz_scal.p, p->lz_part.p, p->lz_vec.p, n, std::max(p->lz_cap_k, 2)};
    double* x = evec_dev;
    double* hx = ws.vec;
    double* r = ws.vec + n;
    const int lz_prec = p->precision;
    tk_status st;
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
        // split precision: FP64 correction steps
        for (int it = 0; it < cfg->refine && lz_prec != TK_PREC_FP64 && rn > cfg->tol; ++it) {
            const int cg_iters = 16;
            if ((st = correction_step(p, ws, x, r, E, cg_iters, lz_prec, s)) != TK_OK) return st;
            matvecs += cg_iters;
            if ((st = fp64_residual(p, ws, x, hx, r, &E, &rn, s)) != TK_OK) return st;
            ++fp64_matvecs;
            ++matvecs;
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
