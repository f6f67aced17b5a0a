// Dense LU factorization with partial pivoting (FP64) and its solves: the
// pivoted factorization behind the cortical-mapping systems, whose KKT
// matrices are symmetric indefinite (OpenMEEG solves them through an SVD
// pseudo-inverse and LAPACK inverses, assembleHeadMat.cpp:168-323).
//
// Right-looking and blocked by NB columns: each column of a panel is one
// pivot launch (first row of largest magnitude, LAPACK's idamax rule, and the
// swap of the two whole rows) and one update launch (multipliers below the
// pivot, rank-1 update of the panel's later columns, one thread per row);
// then U12 = L11^-1 A12 (a warp per column) and the trailing update
// A22 -= L21 U12 on the FP64 GEMM.  The row permutation is kept as LAPACK's
// ipiv (0-based) and as the gather order it composes to.  An exact zero pivot
// is reported (OMG_ERR_SINGULAR) and skipped, as LAPACK's dgetrf does.
#include <algorithm>
#include <vector>

#include "handles.h"
#include "omg_internal.h"

namespace omg {

template <typename T>
void gemm(int64_t M, int64_t N, int64_t K, T alpha, const T* A, int64_t lda, bool ta, const T* B, int64_t ldb, bool tb,
          T beta, T* C, int64_t ldc, cudaStream_t s, bool lower = false, int64_t row0 = 0, int64_t col0 = 0);

namespace lu {

constexpr int NB = 64;
constexpr int PIV_THREADS = 1024;

static inline void check(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error(OMG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    count_launch();
}

// Column j: the pivot row p >= j (largest |A(p, j)|, the first one on ties)
// and the swap of rows j and p over all n columns.
__global__ void __launch_bounds__(PIV_THREADS) pivot_kernel(int64_t n, double* A, int64_t lda, int64_t j, int* piv,
                                                            int* err) {
    __shared__ double sv[PIV_THREADS / 32];
    __shared__ int64_t si[PIV_THREADS / 32];
    __shared__ int64_t s_p;
    double best = -1.0;
    int64_t bi = n;
    for (int64_t i = j + threadIdx.x; i < n; i += blockDim.x) {
        const double v = fabs(A[i + j * lda]);
        if (v > best) {
            best = v;
            bi = i;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) {
            best = ov;
            bi = oi;
        }
    }
    if (lane == 0) {
        sv[warp] = best;
        si[warp] = bi;
    }
    __syncthreads();
    if (warp == 0) {
        best = lane < PIV_THREADS / 32 ? sv[lane] : -1.0;
        bi = lane < PIV_THREADS / 32 ? si[lane] : n;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, best, o);
            const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) {
                best = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            // no finite nonzero candidate (all zero or NaN): keep row j, report
            if (!(best > 0.0) || bi >= n) {
                atomicCAS(err, 0, OMG_ERR_SINGULAR);
                bi = j;
            }
            s_p = bi;
            piv[j] = (int)bi;
        }
    }
    __syncthreads();
    const int64_t p = s_p;
    if (p != j)
        for (int64_t c = threadIdx.x; c < n; c += blockDim.x) {
            const double a = A[j + c * lda];
            A[j + c * lda] = A[p + c * lda];
            A[p + c * lda] = a;
        }
}

// Column j of the panel ending at j1: multipliers l_i = A(i, j) / A(j, j)
// and A(i, c) -= l_i A(j, c) for j < c < j1, one thread per row i > j.
__global__ void panel_update_kernel(int64_t n, double* A, int64_t lda, int64_t j, int64_t j1) {
    const int64_t i = j + 1 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double d = A[j + j * lda];
    if (d == 0.0) return;
    const double l = A[i + j * lda] / d;
    A[i + j * lda] = l;
    for (int64_t c = j + 1; c < j1; ++c) A[i + c * lda] -= l * A[j + c * lda];
}

// X <- T^-1 X for an nb x nb triangle T (nb <= NB) and the ncol columns of X
// (column-major, ldx): lower with unit diagonal (forward) or upper (backward).
// A warp per column; lanes hold rows lane and lane + 32.
template <bool UPPER>
__global__ void __launch_bounds__(256) tri_solve_kernel(int nb, const double* __restrict__ T, int64_t ldt, double* X,
                                                        int64_t ldx, int64_t ncol) {
    __shared__ double sT[NB * NB];   // sT[r + c * NB] = T(r, c)
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
        const int r = e % nb, c = e / nb;
        sT[r + c * NB] = T[r + (int64_t)c * ldt];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t col = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (col >= ncol) return;
    double* x = X + col * ldx;
    double v0 = lane < nb ? x[lane] : 0.0, v1 = lane + 32 < nb ? x[lane + 32] : 0.0;
    if (!UPPER) {
        for (int r = 0; r < nb; ++r) {   // x_r is final; subtract its column below the diagonal
            const double xr = __shfl_sync(0xffffffffu, r < 32 ? v0 : v1, r & 31);
            if (lane > r && lane < nb) v0 -= sT[lane + r * NB] * xr;
            if (lane + 32 > r && lane + 32 < nb) v1 -= sT[lane + 32 + r * NB] * xr;
        }
    } else {
        for (int r = nb - 1; r >= 0; --r) {
            const double d = sT[r + r * NB];
            if (r < 32) {
                if (lane == r) v0 = v0 / d;
            } else if (lane == r - 32) {
                v1 = v1 / d;
            }
            const double xr = __shfl_sync(0xffffffffu, r < 32 ? v0 : v1, r & 31);
            if (lane < r) v0 -= sT[lane + r * NB] * xr;
            if (lane + 32 < r) v1 -= sT[lane + 32 + r * NB] * xr;
        }
    }
    if (lane < nb) x[lane] = v0;
    if (lane + 32 < nb) x[lane + 32] = v1;
}

// Y(i, c) = X(perm[i], c): the rows of X in pivoted order.
__global__ void permute_rows_kernel(int64_t n, int64_t ncol, const int64_t* __restrict__ perm,
                                    const double* __restrict__ X, int64_t ldx, double* Y, int64_t ldy) {
    const int64_t c = blockIdx.y;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        Y[i + c * ldy] = X[perm[i] + c * ldx];
}

template <bool UPPER>
static void tri_solve(int nb, const double* T, int64_t ldt, double* X, int64_t ldx, int64_t ncol, cudaStream_t s) {
    if (ncol <= 0 || nb <= 0) return;
    ProfScope prof_("lu_trsm", s);
    tri_solve_kernel<UPPER><<<(unsigned)((ncol + 7) / 8), 256, 0, s>>>(nb, T, ldt, X, ldx, ncol);
    check("lu tri solve");
}

}  // namespace lu

// In place: A (n x n, column-major, lda) = P L U.  ipiv (device, n ints):
// row j was swapped with row ipiv[j] at step j.  perm (host, n): row i of
// P^T A is row perm[i] of A.  Returns 0 or OMG_ERR_SINGULAR (read back here).
void lu_factor(int64_t n, double* A, int64_t lda, int* ipiv, std::vector<int64_t>& perm, int* err, cudaStream_t s) {
    if (n <= 0) return;
    if (n > INT32_MAX) throw Error(OMG_ERR_UNSUPPORTED, "LU: matrix too large");
    ProfScope prof_("lu_factor", s);
    for (int64_t j0 = 0; j0 < n; j0 += lu::NB) {
        const int64_t jb = std::min<int64_t>(lu::NB, n - j0), j1 = j0 + jb;
        for (int64_t j = j0; j < j1; ++j) {
            lu::pivot_kernel<<<1, lu::PIV_THREADS, 0, s>>>(n, A, lda, j, ipiv, err);
            lu::check("lu pivot");
            if (j + 1 < n) {
                lu::panel_update_kernel<<<(unsigned)((n - j - 1 + 255) / 256), 256, 0, s>>>(n, A, lda, j, j1);
                lu::check("lu panel");
            }
        }
        if (j1 < n) {
            lu::tri_solve<false>((int)jb, A + j0 + j0 * lda, lda, A + j0 + j1 * lda, lda, n - j1, s);
            gemm<double>(n - j1, n - j1, jb, -1.0, A + j1 + j0 * lda, lda, false, A + j0 + j1 * lda, lda, false, 1.0,
                         A + j1 + j1 * lda, lda, s);
        }
    }
    std::vector<int> hp((size_t)n);
    OMG_CUDA(cudaMemcpyAsync(hp.data(), ipiv, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, s));
    OMG_CUDA(cudaStreamSynchronize(s));
    perm.resize((size_t)n);
    for (int64_t i = 0; i < n; ++i) perm[(size_t)i] = i;
    for (int64_t j = 0; j < n; ++j) std::swap(perm[(size_t)j], perm[(size_t)hp[(size_t)j]]);
}

// B (n x nrhs, ldb) <- A^-1 B from lu_factor's output; perm_dev: perm on the device.
void lu_solve(int64_t n, int64_t nrhs, const double* LU, int64_t lda, const int64_t* perm_dev, double* B, int64_t ldb,
              cudaStream_t s) {
    if (n <= 0 || nrhs <= 0) return;
    ProfScope prof_("lu_solve", s);
    DevBuf tmp((size_t)n * nrhs * sizeof(double), s);
    double* Y = tmp.as<double>();
    dim3 grid((unsigned)std::min<int64_t>((n + 255) / 256, 1024), (unsigned)nrhs);
    if (nrhs > 65535) throw Error(OMG_ERR_UNSUPPORTED, "LU solve: too many right-hand sides");
    lu::permute_rows_kernel<<<grid, 256, 0, s>>>(n, nrhs, perm_dev, B, ldb, Y, n);
    lu::check("lu permute");
    for (int64_t b0 = 0; b0 < n; b0 += lu::NB) {   // L y = P^T b
        const int64_t nb = std::min<int64_t>(lu::NB, n - b0), b1 = b0 + nb;
        lu::tri_solve<false>((int)nb, LU + b0 + b0 * lda, lda, Y + b0, n, nrhs, s);
        if (b1 < n) gemm<double>(n - b1, nrhs, nb, -1.0, LU + b1 + b0 * lda, lda, false, Y + b0, n, false, 1.0, Y + b1, n, s);
    }
    const int64_t nblk = (n + lu::NB - 1) / lu::NB;
    for (int64_t bi = nblk - 1; bi >= 0; --bi) {   // U x = y
        const int64_t b0 = bi * lu::NB, nb = std::min<int64_t>(lu::NB, n - b0);
        lu::tri_solve<true>((int)nb, LU + b0 + b0 * lda, lda, Y + b0, n, nrhs, s);
        if (b0 > 0) gemm<double>(b0, nrhs, nb, -1.0, LU + b0 * lda, lda, false, Y + b0, n, false, 1.0, Y, n, s);
    }
    OMG_CUDA(cudaMemcpy2DAsync(B, ldb * 8, Y, n * 8, n * 8, nrhs, cudaMemcpyDeviceToDevice, s));
}

}  // namespace omg

// Test hook (not part of the public header): B <- A^-1 B through lu_factor /
// lu_solve (device pointers, column-major, A overwritten by its factors).
extern "C" int omg_internal_lu_solve(int64_t n, int64_t nrhs, double* A, double* B, int* err) {
    try {
        cudaStream_t s = 0;
        DevBuf ipiv((size_t)std::max<int64_t>(n, 1) * sizeof(int), s);
        std::vector<int64_t> perm;
        omg::lu_factor(n, A, n, ipiv.as<int>(), perm, err, s);
        std::vector<DevBuf> keep;
        omg::lu_solve(n, nrhs, A, n, upload(keep, perm, s), B, n, s);
        return cudaDeviceSynchronize() == cudaSuccess ? 0 : -2;
    } catch (const omg::Error& e) {
        return e.code;
    }
}
