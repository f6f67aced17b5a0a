// Dense kernels for the head-matrix solve: a register-tiled GEMM (FP64 and
// FP32 CUDA cores), the diagonal-block Cholesky + triangular inverse of the
// quasi-definite LDL^T, and small matrix utilities.
//
// The factorization replaces the reference's packed Bunch-Kaufman inverse
// (SymMatrix::invert / solveLin -> DSPTRF/DSPTRI/DSPTRS,
// OpenMEEGMaths/include/symmatrix.h:280-300, src/symmatrix.cpp:133-152).  The
// head matrix in [triangles | vertices] order is symmetric quasi-definite:
// its triangle block is positive definite (single-layer operators) and the
// vertex Schur complement negative definite, so HM = L diag(+I, -I) L^T exists
// without pivoting.  A pivot of the wrong sign is reported, never hidden.
#include <algorithm>
#include <cstdint>

#include "omg_internal.h"

namespace omg {

static inline void check(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error(OMG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    count_launch();
}
static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// ---------------------------------------------------------------------------
// C = alpha * op(A) * op(B) + beta * C (column-major).  LOWER restricts the
// output to entries with global row >= global column (row0/col0 give the
// tile's offsets in the full matrix) and skips tiles strictly above it.
// ---------------------------------------------------------------------------
template <typename T, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    gemm_kernel(int64_t M, int64_t N, int64_t K, T alpha, const T* __restrict__ A, int64_t lda, int ta,
                const T* __restrict__ B, int64_t ldb, int tb, T beta, T* C, int64_t ldc, int lower, int64_t row0,
                int64_t col0) {
    constexpr int NT = (BM / TM) * (BN / TN);
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN + 1];
    const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
    if (lower && (col0 + n0) > (row0 + m0 + BM - 1)) return;
    const int tid = threadIdx.x;
    const int tx = tid % (BN / TN), ty = tid / (BN / TN);
    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = T(0);
    for (int64_t k0 = 0; k0 < K; k0 += BK) {
        // A tile: op(A)(m, k)
        for (int e = tid; e < BM * BK; e += NT) {
            int i, k;
            if (!ta) { i = e % BM; k = e / BM; } else { k = e % BK; i = e / BK; }
            const int64_t gi = m0 + i, gk = k0 + k;
            T v = T(0);
            if (gi < M && gk < K) v = ta ? A[gk + gi * lda] : A[gi + gk * lda];
            As[k][i] = v;
        }
        for (int e = tid; e < BN * BK; e += NT) {
            int j, k;
            if (tb) { j = e % BN; k = e / BN; } else { k = e % BK; j = e / BK; }
            const int64_t gj = n0 + j, gk = k0 + k;
            T v = T(0);
            if (gj < N && gk < K) v = tb ? B[gj + gk * ldb] : B[gk + gj * ldb];
            Bs[k][j] = v;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < BK; ++k) {
            T a[TM], b[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) a[i] = As[k][ty * TM + i];
#pragma unroll
            for (int j = 0; j < TN; ++j) b[j] = Bs[k][tx * TN + j];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < TN; ++j) {
        const int64_t gj = n0 + tx * TN + j;
        if (gj >= N) continue;
#pragma unroll
        for (int i = 0; i < TM; ++i) {
            const int64_t gi = m0 + ty * TM + i;
            if (gi >= M) continue;
            if (lower && row0 + gi < col0 + gj) continue;
            T* c = C + gi + gj * ldc;
            *c = (beta == T(0)) ? alpha * acc[i][j] : alpha * acc[i][j] + beta * *c;
        }
    }
}

template <typename T>
void gemm(int64_t M, int64_t N, int64_t K, T alpha, const T* A, int64_t lda, bool ta, const T* B, int64_t ldb, bool tb,
          T beta, T* C, int64_t ldc, cudaStream_t s, bool lower = false, int64_t row0 = 0, int64_t col0 = 0) {
    if (M <= 0 || N <= 0) return;
    ProfScope prof_(sizeof(T) == 8 ? "gemm_f64" : "gemm_f32", s);
    constexpr bool dbl = sizeof(T) == 8;
    // Large tiles for big products; 32x32 tiles when the big-tile grid would
    // leave most of the 152 SMs idle (block-sized solve steps).
    constexpr int BM = dbl ? 64 : 128, BN = dbl ? 64 : 128, BK = 8, TM = dbl ? 4 : 8, TN = dbl ? 4 : 8;
    const int64_t big_ctas = ((N + BN - 1) / BN) * ((M + BM - 1) / BM);
    if (big_ctas < 152 && (M > 32 || N > 32)) {
        dim3 grid(nblk(N, 32), nblk(M, 32));
        if (grid.y > 65535) throw Error(OMG_ERR_UNSUPPORTED, "GEMM too tall");
        gemm_kernel<T, 32, 32, 8, 2, 2><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, ta ? 1 : 0, B, ldb, tb ? 1 : 0,
                                                          beta, C, ldc, lower ? 1 : 0, row0, col0);
        check("gemm");
        return;
    }
    dim3 grid(nblk(N, BN), nblk(M, BM));
    if (grid.y > 65535) throw Error(OMG_ERR_UNSUPPORTED, "GEMM too tall");
    gemm_kernel<T, BM, BN, BK, TM, TN><<<grid, (BM / TM) * (BN / TN), 0, s>>>(
        M, N, K, alpha, A, lda, ta ? 1 : 0, B, ldb, tb ? 1 : 0, beta, C, ldc, lower ? 1 : 0, row0, col0);
    check("gemm");
}
template void gemm<double>(int64_t, int64_t, int64_t, double, const double*, int64_t, bool, const double*, int64_t,
                           bool, double, double*, int64_t, cudaStream_t, bool, int64_t, int64_t);
template void gemm<float>(int64_t, int64_t, int64_t, float, const float*, int64_t, bool, const float*, int64_t, bool,
                          float, float*, int64_t, cudaStream_t, bool, int64_t, int64_t);

// ---------------------------------------------------------------------------
// Diagonal block: lower Cholesky in shared memory, then L^-1 (row by row).
// A (n x n, lower read) is overwritten by L; Linv (n x n) receives L^-1 with
// zeros above the diagonal.  A non-positive pivot sets *err (with the global
// column in *err_col) and is replaced by 1 so the launch completes.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(512) potrf_trinv_kernel(T* A, int64_t lda, int n, T* Linv, int ldi, int* err,
                                                          int64_t* err_col, int64_t col_offset) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T* L = reinterpret_cast<T*>(smraw);   // n x n, column-major, ld = n
    T* X = L + n * n;                     // n x n inverse
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int e = tid; e < n * n; e += nt) {
        const int i = e % n, j = e / n;
        L[e] = (i >= j) ? A[i + j * lda] : T(0);
        X[e] = T(0);
    }
    __syncthreads();
    for (int j = 0; j < n; ++j) {
        if (tid == 0) {
            T d = L[j + j * n];
            if (!(d > T(0))) {
                if (atomicCAS(err, 0, -3 /* OMG_ERR_NOT_DEFINITE */) == 0) *err_col = col_offset + j;
                d = T(1);
            }
            L[j + j * n] = sqrt(d);
        }
        __syncthreads();
        const T djj = L[j + j * n];
        for (int i = j + 1 + tid; i < n; i += nt) L[i + j * n] /= djj;
        __syncthreads();
        const int m = n - j - 1;
        for (int e = tid; e < m * m; e += nt) {
            const int r = j + 1 + e % m, c = j + 1 + e / m;
            if (r >= c) L[r + c * n] -= L[r + j * n] * L[c + j * n];
        }
        __syncthreads();
    }
    // X = L^-1: row i depends on rows < i.
    for (int i = 0; i < n; ++i) {
        const T inv = T(1) / L[i + i * n];
        for (int c = tid; c <= i; c += nt) {
            T s = (c == i) ? T(1) : T(0);
            for (int k = c; k < i; ++k) s -= L[i + k * n] * X[k + c * n];
            X[i + c * n] = s * inv;
        }
        __syncthreads();
    }
    for (int e = tid; e < n * n; e += nt) {
        const int i = e % n, j = e / n;
        if (i >= j) A[i + j * lda] = L[e];
        Linv[i + j * ldi] = X[e];
    }
}

template <typename T>
void potrf_trinv(T* A, int64_t lda, int n, T* Linv, int ldi, int* err, int64_t* err_col, int64_t col_offset,
                 cudaStream_t s) {
    ProfScope prof_("potrf_trinv", s);
    const size_t sm = 2 * (size_t)n * n * sizeof(T);
    if (sm > 227 * 1024) throw Error(OMG_ERR_INVALID, "diagonal block too large for shared memory");
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(potrf_trinv_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        attr = true;
    }
    potrf_trinv_kernel<T><<<1, 512, sm, s>>>(A, lda, n, Linv, ldi, err, err_col, col_offset);
    check("potrf_trinv");
}
template void potrf_trinv<double>(double*, int64_t, int, double*, int, int*, int64_t*, int64_t, cudaStream_t);
template void potrf_trinv<float>(float*, int64_t, int, float*, int, int*, int64_t*, int64_t, cudaStream_t);

// ---------------------------------------------------------------------------
// Utilities
// ---------------------------------------------------------------------------
template <typename T>
__global__ void negate_lower_kernel(T* A, int64_t lda, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int64_t j = blockIdx.y; j <= i; j += gridDim.y) A[i + j * lda] = -A[i + j * lda];
}
template <typename T>
void negate_lower(T* A, int64_t lda, int64_t n, cudaStream_t s) {
    ProfScope prof_("negate_lower", s);
    if (n <= 0) return;
    dim3 grid(nblk(n, 256), (unsigned)std::min<int64_t>(n, 32768));
    negate_lower_kernel<T><<<grid, 256, 0, s>>>(A, lda, n);
    check("negate_lower");
}
template void negate_lower<double>(double*, int64_t, int64_t, cudaStream_t);
template void negate_lower<float>(float*, int64_t, int64_t, cudaStream_t);

template <typename Tin, typename Tout>
__global__ void copy_convert_kernel(int64_t m, int64_t n, const Tin* __restrict__ a, int64_t lda, Tout* b, int64_t ldb,
                                    int lower, Tout scale) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= m) return;
    for (int64_t j = blockIdx.y; j < n; j += gridDim.y) {
        if (lower && i < j) continue;
        b[i + j * ldb] = (Tout)a[i + j * lda] * scale;
    }
}
template <typename Tin, typename Tout>
void copy_convert(int64_t m, int64_t n, const Tin* a, int64_t lda, Tout* b, int64_t ldb, bool lower, Tout scale,
                  cudaStream_t s) {
    ProfScope prof_("copy_convert", s);
    if (m <= 0 || n <= 0) return;
    dim3 grid(nblk(m, 256), (unsigned)std::min<int64_t>(n, 32768));
    copy_convert_kernel<Tin, Tout><<<grid, 256, 0, s>>>(m, n, a, lda, b, ldb, lower ? 1 : 0, scale);
    check("copy_convert");
}
template void copy_convert<double, double>(int64_t, int64_t, const double*, int64_t, double*, int64_t, bool, double,
                                           cudaStream_t);
template void copy_convert<double, float>(int64_t, int64_t, const double*, int64_t, float*, int64_t, bool, float,
                                          cudaStream_t);
template void copy_convert<float, double>(int64_t, int64_t, const float*, int64_t, double*, int64_t, bool, double,
                                          cudaStream_t);
template void copy_convert<float, float>(int64_t, int64_t, const float*, int64_t, float*, int64_t, bool, float,
                                         cudaStream_t);

// Mirror the lower triangle into the upper one (tiled transpose).
__global__ void symmetrize_kernel(double* A, int64_t lda, int64_t n) {
    __shared__ double tile[32][33];
    const int64_t bi = blockIdx.y, bj = blockIdx.x;   // tile row / col
    if (bj > bi) return;
    const int64_t r0 = bi * 32, c0 = bj * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int64_t r = r0 + threadIdx.x, c = c0 + k;
        if (r < n && c < n) tile[k][threadIdx.x] = A[r + c * lda];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int64_t r = c0 + threadIdx.x, c = r0 + k;   // destination (r, c) with r < c
        if (r < n && c < n && r < c) A[r + c * lda] = tile[threadIdx.x][k];
    }
}
void symmetrize(double* A, int64_t lda, int64_t n, cudaStream_t s) {
    ProfScope prof_("symmetrize", s);
    const int64_t nt = (n + 31) / 32;
    if (nt > 65535) throw Error(OMG_ERR_UNSUPPORTED, "matrix too large to symmetrize");
    dim3 grid((unsigned)nt, (unsigned)nt);
    symmetrize_kernel<<<grid, dim3(32, 8), 0, s>>>(A, lda, n);
    check("symmetrize");
}

// Negate rows [r0, r1) of an m x n matrix (applies D = diag(+I, -I)).
template <typename T>
__global__ void negate_rows_kernel(T* B, int64_t ldb, int64_t r0, int64_t r1, int64_t n) {
    const int64_t i = r0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= r1) return;
    for (int64_t j = blockIdx.y; j < n; j += gridDim.y) B[i + j * ldb] = -B[i + j * ldb];
}
template <typename T>
void negate_rows(T* B, int64_t ldb, int64_t r0, int64_t r1, int64_t n, cudaStream_t s) {
    ProfScope prof_("negate_rows", s);
    if (r1 <= r0 || n <= 0) return;
    dim3 grid(nblk(r1 - r0, 256), (unsigned)std::min<int64_t>(n, 32768));
    negate_rows_kernel<T><<<grid, 256, 0, s>>>(B, ldb, r0, r1, n);
    check("negate_rows");
}
template void negate_rows<double>(double*, int64_t, int64_t, int64_t, int64_t, cudaStream_t);
template void negate_rows<float>(float*, int64_t, int64_t, int64_t, int64_t, cudaStream_t);

// Column norms (squared sums) of an m x n FP64 matrix: one CTA per column.
__global__ void col_norms_kernel(int64_t m, const double* __restrict__ A, int64_t lda, double* out) {
    __shared__ double red[256];
    const int64_t j = blockIdx.x;
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
        const double v = A[i + j * lda];
        s += v * v;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[j] = sqrt(red[0]);
}
void col_norms(int64_t m, int64_t n, const double* A, int64_t lda, double* out, cudaStream_t s) {
    ProfScope prof_("col_norms", s);
    if (n <= 0) return;
    col_norms_kernel<<<(unsigned)n, 256, 0, s>>>(m, A, lda, out);
    check("col_norms");
}

// x += d (FP64 accumulate of an FP32 correction), elementwise on m x n.
__global__ void axpy_f32_kernel(int64_t m, int64_t n, const float* __restrict__ d, int64_t ldd, double* x,
                                int64_t ldx, const double* __restrict__ colscale) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= m) return;
    for (int64_t j = blockIdx.y; j < n; j += gridDim.y)
        x[i + j * ldx] += (double)d[i + j * ldd] * (colscale ? colscale[j] : 1.0);
}
void axpy_f32(int64_t m, int64_t n, const float* d, int64_t ldd, double* x, int64_t ldx, const double* colscale,
              cudaStream_t s) {
    ProfScope prof_("axpy_f32", s);
    dim3 grid(nblk(m, 256), (unsigned)std::min<int64_t>(n, 32768));
    axpy_f32_kernel<<<grid, 256, 0, s>>>(m, n, d, ldd, x, ldx, colscale);
    check("axpy_f32");
}

// b32 = r / scale_j (column scaling before the FP32 correction solve).
__global__ void scale_to_f32_kernel(int64_t m, int64_t n, const double* __restrict__ r, int64_t ldr, float* b,
                                    int64_t ldb, const double* __restrict__ colnorm, double* colscale) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= m) return;
    for (int64_t j = blockIdx.y; j < n; j += gridDim.y) {
        const double sc = colnorm[j] > 0 ? colnorm[j] : 1.0;
        b[i + j * ldb] = (float)(r[i + j * ldr] / sc);
        if (i == 0) colscale[j] = sc;
    }
}
void scale_to_f32(int64_t m, int64_t n, const double* r, int64_t ldr, float* b, int64_t ldb, const double* colnorm,
                  double* colscale, cudaStream_t s) {
    ProfScope prof_("scale_to_f32", s);
    dim3 grid(nblk(m, 256), (unsigned)std::min<int64_t>(n, 32768));
    scale_to_f32_kernel<<<grid, 256, 0, s>>>(m, n, r, ldr, b, ldb, colnorm, colscale);
    check("scale_to_f32");
}

}  // namespace omg
