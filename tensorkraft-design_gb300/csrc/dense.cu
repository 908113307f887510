// dense.cu -- the dense factorisations of LinAlgBackend on the device:
// svd_truncated, eigh_lowest and qr (tk-linalg/src/traits.rs:63-148), with
// the conventions of the reference's faer backend (device/faer.rs:127-325):
// singular values descending, rank = count of sigma >= cutoff * sigma_max up to
// max_rank, truncation error = sum of the discarded sigma^2, U (m x rank) and
// Vt (rank x n) row-major; eigenvalues ascending with eigenvectors as the
// columns of an (n x k) row-major matrix; thin Q (m x k) and R (k x n),
// k = min(m, n), row-major.  The factorisations themselves are cuSOLVER's
// (Jacobi SVD, divide-and-conquer symmetric eigensolver, Householder QR);
// the strided gathers and the row-major outputs are kernels of this file.
#include <cuda_runtime.h>
#include <cuComplex.h>
#include <cusolverDn.h>

#include <algorithm>
#include <string>
#include <vector>

#include "tk_internal.hpp"

namespace tk {
tk_status cuda_fail(const char* op, cudaError_t e);

namespace {

// dst (column-major m x n, ld m) = src(i, j) = src[i * rs + j * cs]
__global__ void gather_colmajor_kernel(const double* __restrict__ src, int64_t rs, int64_t cs, int64_t m, int64_t n,
                                       double* __restrict__ dst) {
    const int64_t total = m * n;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % m, j = e / m;
        dst[e] = src[i * rs + j * cs];
    }
}

// dst row-major (rows x cols) = src column-major (ld) element (i, j), or its
// transpose element (j, i) when `transpose`; below-diagonal zero when `upper`.
__global__ void to_rowmajor_kernel(const double* __restrict__ src, int64_t ld, int64_t rows, int64_t cols,
                                   bool transpose, bool upper, double* __restrict__ dst) {
    const int64_t total = rows * cols;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e / cols, j = e % cols;
        double v = transpose ? src[j + i * ld] : src[i + j * ld];
        if (upper && j < i) v = 0.0;
        dst[e] = v;
    }
}

// dst (column-major m x n complex, ld m) = element (i, j) of a planar strided
// matrix, conjugated when `conj`.
__global__ void gather_cplx_colmajor_kernel(const double* __restrict__ re, const double* __restrict__ im, int64_t rs,
                                            int64_t cs, int64_t m, int64_t n, bool conj,
                                            cuDoubleComplex* __restrict__ dst) {
    const int64_t total = m * n;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % m, j = e / m, o = i * rs + j * cs;
        dst[e] = make_cuDoubleComplex(re[o], conj ? -im[o] : im[o]);
    }
}

// planar row-major (rows x cols) = complex column-major (ld) element (i, j),
// or the conjugate transpose element (j, i)^* when `adjoint`; below-diagonal
// zero when `upper`.
__global__ void cplx_to_rowmajor_kernel(const cuDoubleComplex* __restrict__ src, int64_t ld, int64_t rows,
                                        int64_t cols, bool adjoint, bool upper, double* __restrict__ re,
                                        double* __restrict__ im) {
    const int64_t total = rows * cols;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e / cols, j = e % cols;
        cuDoubleComplex v = adjoint ? src[j + i * ld] : src[i + j * ld];
        if (adjoint) v.y = -v.y;
        if (upper && j < i) v = make_cuDoubleComplex(0.0, 0.0);
        re[e] = v.x;
        im[e] = v.y;
    }
}

int grid_for(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8)); }

struct Dev {
    std::vector<void*> ptrs;
    ~Dev() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    cudaError_t alloc(T** p, size_t count) {
        cudaError_t e = cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(count, 1));
        if (e == cudaSuccess) ptrs.push_back(*p);
        return e;
    }
};

tk_status solver_fail(const char* op, cusolverStatus_t st) {
    set_error(std::string(op) + ": cuSOLVER status " + std::to_string((int)st));
    return TK_ERR_CUDA;
}

struct Guard {
    int prev = -1;
    bool ok = false;
    explicit Guard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        ok = (cudaSetDevice(dev) == cudaSuccess);
    }
    ~Guard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

tk_status handle_of(tk_ctx* ctx, cudaStream_t s, cusolverDnHandle_t* h, const char* name) {
    if (!ctx->solver) {
        cusolverDnHandle_t nh = nullptr;
        cusolverStatus_t st = cusolverDnCreate(&nh);
        if (st != CUSOLVER_STATUS_SUCCESS) return solver_fail(name, st);
        ctx->solver = nh;
    }
    *h = (cusolverDnHandle_t)ctx->solver;
    cusolverStatus_t st = cusolverDnSetStream(*h, s);
    return st == CUSOLVER_STATUS_SUCCESS ? TK_OK : solver_fail(name, st);
}

bool mat_ok(const tk_mat* a) { return a && a->data && a->rows > 0 && a->cols > 0; }
bool cmat_ok(const tk_cmat* a) { return a && a->re && a->im && a->rows > 0 && a->cols > 0; }

tk_status check_info(int* dinfo, cudaStream_t s, const char* name) {
    int info = 0;
    cudaError_t e = cudaMemcpyAsync(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(name, e);
    if (info != 0) {
        set_error(std::string(name) + ": cuSOLVER info " + std::to_string(info) +
                  (info > 0 ? " (no convergence)" : " (invalid argument)"));
        return info > 0 ? TK_ERR_UNSUPPORTED : TK_ERR_INVALID_ARG;
    }
    return TK_OK;
}

}  // namespace

void ctx_release_solver(tk_ctx* ctx) {
    if (ctx && ctx->solver) {
        cusolverDnDestroy((cusolverDnHandle_t)ctx->solver);
        ctx->solver = nullptr;
    }
}

}  // namespace tk

using namespace tk;

extern "C" {

tk_status tk_svd_truncated_f64(tk_ctx* ctx, const tk_mat* a, int64_t max_rank, double cutoff, double* u_dev,
                               double* s_host, double* vt_dev, int64_t* rank, double* truncation_error,
                               void* stream) {
    if (!ctx || !mat_ok(a) || !u_dev || !s_host || !vt_dev || !rank || max_rank < 0) {
        set_error("tk_svd_truncated_f64: invalid argument");
        return TK_ERR_INVALID_ARG;
    }
    Guard g(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;
    cusolverDnHandle_t h;
    tk_status st = handle_of(ctx, s, &h, "tk_svd_truncated_f64");
    if (st != TK_OK) return st;
    const int m = (int)a->rows, n = (int)a->cols, k = std::min(m, n);
    Dev d;
    double *A, *S, *U, *V, *work;
    int* info;
    cudaError_t e;
    if ((e = d.alloc(&A, (size_t)m * n)) != cudaSuccess || (e = d.alloc(&S, (size_t)k)) != cudaSuccess ||
        (e = d.alloc(&U, (size_t)m * k)) != cudaSuccess || (e = d.alloc(&V, (size_t)n * k)) != cudaSuccess ||
        (e = d.alloc(&info, 1)) != cudaSuccess)
        return cuda_fail("tk_svd_truncated_f64: workspace", e);
    gather_colmajor_kernel<<<grid_for((int64_t)m * n), 256, 0, s>>>(a->data, a->row_stride, a->col_stride, m, n, A);
    gesvdjInfo_t params = nullptr;
    cusolverStatus_t cs = cusolverDnCreateGesvdjInfo(&params);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("gesvdj info", cs);
    int lwork = 0;
    cs = cusolverDnDgesvdj_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, 1, m, n, A, m, S, U, m, V, n, &lwork, params);
    if (cs == CUSOLVER_STATUS_SUCCESS && (e = d.alloc(&work, (size_t)lwork)) != cudaSuccess) {
        cusolverDnDestroyGesvdjInfo(params);
        return cuda_fail("tk_svd_truncated_f64: workspace", e);
    }
    if (cs == CUSOLVER_STATUS_SUCCESS)
        cs = cusolverDnDgesvdj(h, CUSOLVER_EIG_MODE_VECTOR, 1, m, n, A, m, S, U, m, V, n, work, lwork, info, params);
    cusolverDnDestroyGesvdjInfo(params);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("gesvdj", cs);
    if ((st = check_info(info, s, "tk_svd_truncated_f64")) != TK_OK) return st;
    std::vector<double> sv((size_t)k);
    if ((e = cudaMemcpy(sv.data(), S, sizeof(double) * k, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_fail("tk_svd_truncated_f64", e);
    // descending order (cuSOLVER's Jacobi SVD returns it so); checked, not assumed
    for (int i = 1; i < k; ++i)
        if (sv[i] > sv[i - 1]) {
            set_error("tk_svd_truncated_f64: singular values not in descending order");
            return TK_ERR_CUDA;
        }
    const double thr = cutoff * (k > 0 ? sv[0] : 0.0);
    int r = 0;
    while (r < k && r < max_rank && !(sv[r] < thr)) ++r;
    double terr = 0.0;
    for (int i = r; i < k; ++i) terr += sv[i] * sv[i];
    for (int i = 0; i < r; ++i) s_host[i] = sv[i];
    *rank = r;
    if (truncation_error) *truncation_error = terr;
    if (r > 0) {
        to_rowmajor_kernel<<<grid_for((int64_t)m * r), 256, 0, s>>>(U, m, m, r, false, false, u_dev);
        to_rowmajor_kernel<<<grid_for((int64_t)r * n), 256, 0, s>>>(V, n, r, n, true, false, vt_dev);
    }
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail("tk_svd_truncated_f64", e);
    return TK_OK;
}

tk_status tk_eigh_lowest_f64(tk_ctx* ctx, const tk_mat* a, int64_t k, double* evals_host, double* evecs_dev,
                             void* stream) {
    if (!ctx || !mat_ok(a) || a->rows != a->cols || !evals_host || !evecs_dev || k < 0) {
        set_error("tk_eigh_lowest_f64: invalid argument (a square matrix is required)");
        return TK_ERR_INVALID_ARG;
    }
    const int n = (int)a->rows;
    if (k > n) {  // LinAlgError::EighKTooLarge
        set_error("tk_eigh_lowest_f64: k larger than the matrix dimension");
        return TK_ERR_INVALID_ARG;
    }
    Guard g(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;
    cusolverDnHandle_t h;
    tk_status st = handle_of(ctx, s, &h, "tk_eigh_lowest_f64");
    if (st != TK_OK) return st;
    Dev d;
    double *A, *W, *work;
    int* info;
    cudaError_t e;
    if ((e = d.alloc(&A, (size_t)n * n)) != cudaSuccess || (e = d.alloc(&W, (size_t)n)) != cudaSuccess ||
        (e = d.alloc(&info, 1)) != cudaSuccess)
        return cuda_fail("tk_eigh_lowest_f64: workspace", e);
    gather_colmajor_kernel<<<grid_for((int64_t)n * n), 256, 0, s>>>(a->data, a->row_stride, a->col_stride, n, n, A);
    int lwork = 0;
    cusolverStatus_t cs =
        cusolverDnDsyevd_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, A, n, W, &lwork);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("syevd", cs);
    if ((e = d.alloc(&work, (size_t)lwork)) != cudaSuccess) return cuda_fail("tk_eigh_lowest_f64: workspace", e);
    cs = cusolverDnDsyevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, A, n, W, work, lwork, info);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("syevd", cs);
    if ((st = check_info(info, s, "tk_eigh_lowest_f64")) != TK_OK) return st;
    if (k > 0) {
        if ((e = cudaMemcpy(evals_host, W, sizeof(double) * k, cudaMemcpyDeviceToHost)) != cudaSuccess)
            return cuda_fail("tk_eigh_lowest_f64", e);
        to_rowmajor_kernel<<<grid_for((int64_t)n * k), 256, 0, s>>>(A, n, n, k, false, false, evecs_dev);
    }
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail("tk_eigh_lowest_f64", e);
    return TK_OK;
}

tk_status tk_eigh_batched_f64(tk_ctx* ctx, int64_t n, int64_t batch, const double* a_host, double* w_host,
                              double* z_host) {
    if (!ctx || n <= 0 || batch < 0 || (batch > 0 && (!a_host || !w_host || !z_host))) {
        set_error("tk_eigh_batched_f64: invalid argument");
        return TK_ERR_INVALID_ARG;
    }
    if (batch == 0) return TK_OK;
    Guard g(ctx->device);
    cudaStream_t s = 0;
    cusolverDnHandle_t h;
    tk_status st = handle_of(ctx, s, &h, "tk_eigh_batched_f64");
    if (st != TK_OK) return st;
    cusolverDnParams_t params = nullptr;
    cusolverStatus_t cs = cusolverDnCreateParams(&params);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("tk_eigh_batched_f64: params", cs);
    struct ParamsFree {
        cusolverDnParams_t p;
        ~ParamsFree() { cusolverDnDestroyParams(p); }
    } pf{params};
    const size_t nn = (size_t)n * (size_t)n * (size_t)batch;
    Dev d;
    double *A, *W;
    int* info;
    cudaError_t e;
    if ((e = d.alloc(&A, nn)) != cudaSuccess || (e = d.alloc(&W, (size_t)n * batch)) != cudaSuccess ||
        (e = d.alloc(&info, (size_t)batch)) != cudaSuccess)
        return cuda_fail("tk_eigh_batched_f64: workspace", e);
    if ((e = cudaMemcpyAsync(A, a_host, sizeof(double) * nn, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail("tk_eigh_batched_f64: upload", e);
    size_t wdev = 0, whost = 0;
    cs = cusolverDnXsyevBatched_bufferSize(h, params, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, CUDA_R_64F,
                                           A, n, CUDA_R_64F, W, CUDA_R_64F, &wdev, &whost, batch);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("syevBatched buffer size", cs);
    uint8_t* work = nullptr;
    if ((e = d.alloc(&work, wdev)) != cudaSuccess) return cuda_fail("tk_eigh_batched_f64: workspace", e);
    std::vector<uint8_t> hwork(std::max<size_t>(whost, 1));
    cs = cusolverDnXsyevBatched(h, params, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, CUDA_R_64F, A, n,
                                CUDA_R_64F, W, CUDA_R_64F, work, wdev, hwork.data(), whost, info, batch);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("syevBatched", cs);
    std::vector<int> hinfo((size_t)batch);
    if ((e = cudaMemcpyAsync(hinfo.data(), info, sizeof(int) * batch, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(w_host, W, sizeof(double) * n * batch, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(z_host, A, sizeof(double) * nn, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail("tk_eigh_batched_f64: download", e);
    for (int64_t b = 0; b < batch; ++b)
        if (hinfo[(size_t)b] != 0) {
            set_error("tk_eigh_batched_f64: cuSOLVER info " + std::to_string(hinfo[(size_t)b]) + " for matrix " +
                      std::to_string(b));
            return hinfo[(size_t)b] > 0 ? TK_ERR_UNSUPPORTED : TK_ERR_INVALID_ARG;
        }
    return TK_OK;
}

tk_status tk_qr_f64(tk_ctx* ctx, const tk_mat* a, double* q_dev, double* r_dev, void* stream) {
    if (!ctx || !mat_ok(a) || !q_dev || !r_dev) {
        set_error("tk_qr_f64: invalid argument");
        return TK_ERR_INVALID_ARG;
    }
    Guard g(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;
    cusolverDnHandle_t h;
    tk_status st = handle_of(ctx, s, &h, "tk_qr_f64");
    if (st != TK_OK) return st;
    const int m = (int)a->rows, n = (int)a->cols, k = std::min(m, n);
    Dev d;
    double *A, *tau, *work;
    int* info;
    cudaError_t e;
    if ((e = d.alloc(&A, (size_t)m * n)) != cudaSuccess || (e = d.alloc(&tau, (size_t)k)) != cudaSuccess ||
        (e = d.alloc(&info, 1)) != cudaSuccess)
        return cuda_fail("tk_qr_f64: workspace", e);
    gather_colmajor_kernel<<<grid_for((int64_t)m * n), 256, 0, s>>>(a->data, a->row_stride, a->col_stride, m, n, A);
    int lw1 = 0, lw2 = 0;
    cusolverStatus_t cs = cusolverDnDgeqrf_bufferSize(h, m, n, A, m, &lw1);
    if (cs == CUSOLVER_STATUS_SUCCESS) cs = cusolverDnDorgqr_bufferSize(h, m, k, k, A, m, tau, &lw2);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("geqrf/orgqr", cs);
    if ((e = d.alloc(&work, (size_t)std::max(lw1, lw2))) != cudaSuccess) return cuda_fail("tk_qr_f64: workspace", e);
    cs = cusolverDnDgeqrf(h, m, n, A, m, tau, work, std::max(lw1, lw2), info);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("geqrf", cs);
    if ((st = check_info(info, s, "tk_qr_f64")) != TK_OK) return st;
    // R: the upper triangle of the first k rows, before orgqr overwrites A
    to_rowmajor_kernel<<<grid_for((int64_t)k * n), 256, 0, s>>>(A, m, k, n, false, true, r_dev);
    cs = cusolverDnDorgqr(h, m, k, k, A, m, tau, work, std::max(lw1, lw2), info);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("orgqr", cs);
    if ((st = check_info(info, s, "tk_qr_f64")) != TK_OK) return st;
    to_rowmajor_kernel<<<grid_for((int64_t)m * k), 256, 0, s>>>(A, m, m, k, false, false, q_dev);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail("tk_qr_f64", e);
    return TK_OK;
}

// ---- complex (C64) factorisations: planar in, planar out ----------------------

tk_status tk_svd_truncated_c64(tk_ctx* ctx, const tk_cmat* a, int64_t max_rank, double cutoff, double* u_re,
                               double* u_im, double* s_host, double* vt_re, double* vt_im, int64_t* rank,
                               double* truncation_error, void* stream) {
    if (!ctx || !cmat_ok(a) || !u_re || !u_im || !s_host || !vt_re || !vt_im || !rank || max_rank < 0) {
        set_error("tk_svd_truncated_c64: invalid argument");
        return TK_ERR_INVALID_ARG;
    }
    Guard g(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;
    cusolverDnHandle_t h;
    tk_status st = handle_of(ctx, s, &h, "tk_svd_truncated_c64");
    if (st != TK_OK) return st;
    const int m = (int)a->rows, n = (int)a->cols, k = std::min(m, n);
    Dev d;
    cuDoubleComplex *A, *U, *V, *work;
    double* S;
    int* info;
    cudaError_t e;
    if ((e = d.alloc(&A, (size_t)m * n)) != cudaSuccess || (e = d.alloc(&S, (size_t)k)) != cudaSuccess ||
        (e = d.alloc(&U, (size_t)m * k)) != cudaSuccess || (e = d.alloc(&V, (size_t)n * k)) != cudaSuccess ||
        (e = d.alloc(&info, 1)) != cudaSuccess)
        return cuda_fail("tk_svd_truncated_c64: workspace", e);
    gather_cplx_colmajor_kernel<<<grid_for((int64_t)m * n), 256, 0, s>>>(a->re, a->im, a->row_stride, a->col_stride, m,
                                                                          n, a->is_conjugated != 0, A);
    gesvdjInfo_t params = nullptr;
    cusolverStatus_t cs = cusolverDnCreateGesvdjInfo(&params);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("gesvdj info", cs);
    int lwork = 0;
    cs = cusolverDnZgesvdj_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, 1, m, n, A, m, S, U, m, V, n, &lwork, params);
    if (cs == CUSOLVER_STATUS_SUCCESS && (e = d.alloc(&work, (size_t)lwork)) != cudaSuccess) {
        cusolverDnDestroyGesvdjInfo(params);
        return cuda_fail("tk_svd_truncated_c64: workspace", e);
    }
    if (cs == CUSOLVER_STATUS_SUCCESS)
        cs = cusolverDnZgesvdj(h, CUSOLVER_EIG_MODE_VECTOR, 1, m, n, A, m, S, U, m, V, n, work, lwork, info, params);
    cusolverDnDestroyGesvdjInfo(params);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("gesvdj (complex)", cs);
    if ((st = check_info(info, s, "tk_svd_truncated_c64")) != TK_OK) return st;
    std::vector<double> sv((size_t)k);
    if ((e = cudaMemcpy(sv.data(), S, sizeof(double) * k, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_fail("tk_svd_truncated_c64", e);
    for (int i = 1; i < k; ++i)
        if (sv[i] > sv[i - 1]) {
            set_error("tk_svd_truncated_c64: singular values not in descending order");
            return TK_ERR_CUDA;
        }
    const double thr = cutoff * (k > 0 ? sv[0] : 0.0);
    int r = 0;
    while (r < k && r < max_rank && !(sv[r] < thr)) ++r;
    double terr = 0.0;
    for (int i = r; i < k; ++i) terr += sv[i] * sv[i];
    for (int i = 0; i < r; ++i) s_host[i] = sv[i];
    *rank = r;
    if (truncation_error) *truncation_error = terr;
    if (r > 0) {
        // A = U S V^H: U (m x r) as is, Vt = V^H (r x n)
        cplx_to_rowmajor_kernel<<<grid_for((int64_t)m * r), 256, 0, s>>>(U, m, m, r, false, false, u_re, u_im);
        cplx_to_rowmajor_kernel<<<grid_for((int64_t)r * n), 256, 0, s>>>(V, n, r, n, true, false, vt_re, vt_im);
    }
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail("tk_svd_truncated_c64", e);
    return TK_OK;
}

tk_status tk_eigh_lowest_c64(tk_ctx* ctx, const tk_cmat* a, int64_t k, double* evals_host, double* evecs_re,
                             double* evecs_im, void* stream) {
    if (!ctx || !cmat_ok(a) || a->rows != a->cols || !evals_host || !evecs_re || !evecs_im || k < 0) {
        set_error("tk_eigh_lowest_c64: invalid argument (a square matrix is required)");
        return TK_ERR_INVALID_ARG;
    }
    const int n = (int)a->rows;
    if (k > n) {  // LinAlgError::EighKTooLarge
        set_error("tk_eigh_lowest_c64: k larger than the matrix dimension");
        return TK_ERR_INVALID_ARG;
    }
    Guard g(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;
    cusolverDnHandle_t h;
    tk_status st = handle_of(ctx, s, &h, "tk_eigh_lowest_c64");
    if (st != TK_OK) return st;
    Dev d;
    cuDoubleComplex *A, *work;
    double* W;
    int* info;
    cudaError_t e;
    if ((e = d.alloc(&A, (size_t)n * n)) != cudaSuccess || (e = d.alloc(&W, (size_t)n)) != cudaSuccess ||
        (e = d.alloc(&info, 1)) != cudaSuccess)
        return cuda_fail("tk_eigh_lowest_c64: workspace", e);
    gather_cplx_colmajor_kernel<<<grid_for((int64_t)n * n), 256, 0, s>>>(a->re, a->im, a->row_stride, a->col_stride, n,
                                                                          n, a->is_conjugated != 0, A);
    int lwork = 0;
    cusolverStatus_t cs =
        cusolverDnZheevd_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, A, n, W, &lwork);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("heevd", cs);
    if ((e = d.alloc(&work, (size_t)lwork)) != cudaSuccess) return cuda_fail("tk_eigh_lowest_c64: workspace", e);
    cs = cusolverDnZheevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, A, n, W, work, lwork, info);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("heevd", cs);
    if ((st = check_info(info, s, "tk_eigh_lowest_c64")) != TK_OK) return st;
    if (k > 0) {
        if ((e = cudaMemcpy(evals_host, W, sizeof(double) * k, cudaMemcpyDeviceToHost)) != cudaSuccess)
            return cuda_fail("tk_eigh_lowest_c64", e);
        cplx_to_rowmajor_kernel<<<grid_for((int64_t)n * k), 256, 0, s>>>(A, n, n, k, false, false, evecs_re, evecs_im);
    }
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail("tk_eigh_lowest_c64", e);
    return TK_OK;
}

tk_status tk_qr_c64(tk_ctx* ctx, const tk_cmat* a, double* q_re, double* q_im, double* r_re, double* r_im,
                    void* stream) {
    if (!ctx || !cmat_ok(a) || !q_re || !q_im || !r_re || !r_im) {
        set_error("tk_qr_c64: invalid argument");
        return TK_ERR_INVALID_ARG;
    }
    Guard g(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;
    cusolverDnHandle_t h;
    tk_status st = handle_of(ctx, s, &h, "tk_qr_c64");
    if (st != TK_OK) return st;
    const int m = (int)a->rows, n = (int)a->cols, k = std::min(m, n);
    Dev d;
    cuDoubleComplex *A, *tau, *work;
    int* info;
    cudaError_t e;
    if ((e = d.alloc(&A, (size_t)m * n)) != cudaSuccess || (e = d.alloc(&tau, (size_t)k)) != cudaSuccess ||
        (e = d.alloc(&info, 1)) != cudaSuccess)
        return cuda_fail("tk_qr_c64: workspace", e);
    gather_cplx_colmajor_kernel<<<grid_for((int64_t)m * n), 256, 0, s>>>(a->re, a->im, a->row_stride, a->col_stride, m,
                                                                          n, a->is_conjugated != 0, A);
    int lw1 = 0, lw2 = 0;
    cusolverStatus_t cs = cusolverDnZgeqrf_bufferSize(h, m, n, A, m, &lw1);
    if (cs == CUSOLVER_STATUS_SUCCESS) cs = cusolverDnZungqr_bufferSize(h, m, k, k, A, m, tau, &lw2);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("geqrf/ungqr", cs);
    if ((e = d.alloc(&work, (size_t)std::max(lw1, lw2))) != cudaSuccess) return cuda_fail("tk_qr_c64: workspace", e);
    cs = cusolverDnZgeqrf(h, m, n, A, m, tau, work, std::max(lw1, lw2), info);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("geqrf (complex)", cs);
    if ((st = check_info(info, s, "tk_qr_c64")) != TK_OK) return st;
    cplx_to_rowmajor_kernel<<<grid_for((int64_t)k * n), 256, 0, s>>>(A, m, k, n, false, true, r_re, r_im);
    cs = cusolverDnZungqr(h, m, k, k, A, m, tau, work, std::max(lw1, lw2), info);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail("ungqr", cs);
    if ((st = check_info(info, s, "tk_qr_c64")) != TK_OK) return st;
    cplx_to_rowmajor_kernel<<<grid_for((int64_t)m * k), 256, 0, s>>>(A, m, m, k, false, false, q_re, q_im);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail("tk_qr_c64", e);
    return TK_OK;
}

}  // extern "C"
