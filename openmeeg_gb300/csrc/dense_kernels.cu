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

// Launch with programmatic dependent launch when `pdl`: the kernel may start while its predecessor on the
// stream finishes and waits for it (griddepcontrol.wait) before it reads that kernel's outputs.
template <typename... KArgs, typename... Args>
static void launch_maybe_pdl(bool pdl, void (*kern)(KArgs...), unsigned grid, unsigned block, size_t smem,
                             cudaStream_t s, Args... args) {
    if (!pdl) {
        kern<<<grid, block, smem, s>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, (KArgs)args...);
}

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

// ---------------------------------------------------------------------------
// Refinement residual R = B - A X with FP64 accuracy on the FP32 pipes.
// A (FP64) and X (FP64) are split into float pairs hi + lo when staged into
// shared memory; each product is formed exactly (TwoProd by FMA, plus the
// cross terms) and accumulated in a compensated pair (TwoSum), the "Dot2"
// scheme of Ogita, Rump and Oishi (SIAM J. Sci. Comput. 26(6), 2005), which
// returns the dot product as if computed in twice the working precision.
// ---------------------------------------------------------------------------
constexpr int RB_M = 64, RB_N = 32, RB_K = 16, RB_TM = 4, RB_TN = 2;   // 256 threads

// Operands arrive pre-split (A = Ah + Al, X = Xh + Xl, float pairs, see
// split_f64), so the inner loop runs on the FP32 pipe only.
__global__ void __launch_bounds__(256) residual_df64_kernel(int64_t M, int64_t N, int64_t K,
                                                           const float* __restrict__ Ahi,
                                                           const float* __restrict__ Alo, int64_t lda,
                                                           const float* __restrict__ Xhi,
                                                           const float* __restrict__ Xlo, int64_t ldx,
                                                           const double* __restrict__ B, int64_t ldb, double* R,
                                                           int64_t ldr) {
    __shared__ float Ah[RB_K][RB_M + 1], Al[RB_K][RB_M + 1];
    __shared__ float Xh[RB_K][RB_N + 1], Xl[RB_K][RB_N + 1];
    const int64_t m0 = (int64_t)blockIdx.y * RB_M, n0 = (int64_t)blockIdx.x * RB_N;
    const int tid = threadIdx.x;
    const int tx = tid % (RB_N / RB_TN), ty = tid / (RB_N / RB_TN);
    float sh[RB_TM][RB_TN], sl[RB_TM][RB_TN];
#pragma unroll
    for (int i = 0; i < RB_TM; ++i)
#pragma unroll
        for (int j = 0; j < RB_TN; ++j) sh[i][j] = sl[i][j] = 0.f;
    for (int64_t k0 = 0; k0 < K; k0 += RB_K) {
        for (int e = tid; e < RB_M * RB_K; e += 256) {
            const int i = e % RB_M, k = e / RB_M;
            const int64_t gi = m0 + i, gk = k0 + k;
            const bool ok = gi < M && gk < K;
            Ah[k][i] = ok ? Ahi[gi + gk * lda] : 0.f;
            Al[k][i] = ok ? Alo[gi + gk * lda] : 0.f;
        }
        for (int e = tid; e < RB_N * RB_K; e += 256) {
            const int k = e % RB_K, j = e / RB_K;
            const int64_t gj = n0 + j, gk = k0 + k;
            const bool ok = gj < N && gk < K;
            Xh[k][j] = ok ? Xhi[gk + gj * ldx] : 0.f;
            Xl[k][j] = ok ? Xlo[gk + gj * ldx] : 0.f;
        }
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < RB_K; ++k) {
            float ah[RB_TM], al[RB_TM], xh[RB_TN], xl[RB_TN];
#pragma unroll
            for (int i = 0; i < RB_TM; ++i) { ah[i] = Ah[k][ty * RB_TM + i]; al[i] = Al[k][ty * RB_TM + i]; }
#pragma unroll
            for (int j = 0; j < RB_TN; ++j) { xh[j] = Xh[k][tx * RB_TN + j]; xl[j] = Xl[k][tx * RB_TN + j]; }
#pragma unroll
            for (int i = 0; i < RB_TM; ++i)
#pragma unroll
                for (int j = 0; j < RB_TN; ++j) {
                    const float p = ah[i] * xh[j];
                    float e = fmaf(ah[i], xh[j], -p);           // exact product error
                    e = fmaf(ah[i], xl[j], e);
                    e = fmaf(al[i], xh[j], e);
                    const float s = sh[i][j] + p;               // TwoSum(sh, p)
                    const float bp = s - sh[i][j];
                    const float t = (sh[i][j] - (s - bp)) + (p - bp);
                    sh[i][j] = s;
                    sl[i][j] += t + e;
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < RB_TN; ++j) {
        const int64_t gj = n0 + tx * RB_TN + j;
        if (gj >= N) continue;
#pragma unroll
        for (int i = 0; i < RB_TM; ++i) {
            const int64_t gi = m0 + ty * RB_TM + i;
            if (gi >= M) continue;
            R[gi + gj * ldr] = B[gi + gj * ldb] - ((double)sh[i][j] + (double)sl[i][j]);
        }
    }
}

void residual_df64(int64_t M, int64_t N, int64_t K, const float* Ahi, const float* Alo, int64_t lda,
                   const float* Xhi, const float* Xlo, int64_t ldx, const double* B, int64_t ldb, double* R,
                   int64_t ldr, cudaStream_t s) {
    if (M <= 0 || N <= 0) return;
    ProfScope prof_("residual_df64", s);
    dim3 grid(nblk(N, RB_N), nblk(M, RB_M));
    residual_df64_kernel<<<grid, 256, 0, s>>>(M, N, K, Ahi, Alo, lda, Xhi, Xlo, ldx, B, ldb, R, ldr);
    check("residual_df64");
}

// FP64 m x n (lda) -> float pair hi = fl(a), lo = fl(a - hi), column-major (ldo).
__global__ void split_f64_kernel(int64_t m, int64_t n, const double* __restrict__ A, int64_t lda, float* H, float* L,
                                 int64_t ldo) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= m) return;
    for (int64_t j = blockIdx.y; j < n; j += gridDim.y) {
        const double v = A[i + j * lda];
        const float h = (float)v;
        H[i + j * ldo] = h;
        L[i + j * ldo] = (float)(v - (double)h);
    }
}
void split_f64(int64_t m, int64_t n, const double* A, int64_t lda, float* H, float* L, int64_t ldo, cudaStream_t s) {
    if (m <= 0 || n <= 0) return;
    ProfScope prof_("split_f64", s);
    dim3 grid(nblk(m, 256), (unsigned)std::min<int64_t>(n, 32768));
    split_f64_kernel<<<grid, 256, 0, s>>>(m, n, A, lda, H, L, ldo);
    check("split_f64");
}

// ---------------------------------------------------------------------------
// Diagonal block Cholesky (lower, right-looking) with the block resident in
// shared memory; thread (r, c-chunk) mapping avoids integer division in the
// update loop.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(512) potrf_kernel(T* A, int64_t lda, int n, int* err, int64_t* err_col,
                                                   int64_t col_offset) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T* L = reinterpret_cast<T*>(smraw);   // n x (n+1) column-major (padded)
    const int ldl = n + 1;
    const int tid = threadIdx.x;
    for (int e = tid; e < n * n; e += 512) {
        const int i = e % n, j = e / n;
        L[i + j * ldl] = (i >= j) ? A[i + j * lda] : T(0);
    }
    __syncthreads();
    const int lane_r = tid % 32, grp = tid / 32;   // 16 groups of 32 rows-threads
    for (int j = 0; j < n; ++j) {
        if (tid == 0) {
            T d = L[j + j * ldl];
            if (!(d > T(0))) {
                if (atomicCAS(err, 0, -3 /* OMG_ERR_NOT_DEFINITE */) == 0) *err_col = col_offset + j;
                d = T(1);
            }
            L[j + j * ldl] = sqrt(d);
        }
        __syncthreads();
        const T inv = T(1) / L[j + j * ldl];
        for (int i = j + 1 + tid; i < n; i += 512) L[i + j * ldl] *= inv;
        __syncthreads();
        // trailing update of columns c in (j, n): group g handles columns c = j+1+g, j+1+g+16, ...
        for (int c = j + 1 + grp; c < n; c += 16) {
            const T lc = L[c + j * ldl];
            for (int r = c + lane_r; r < n; r += 32) L[r + c * ldl] -= L[r + j * ldl] * lc;
        }
        __syncthreads();
    }
    for (int e = tid; e < n * n; e += 512) {
        const int i = e % n, j = e / n;
        if (i >= j) A[i + j * lda] = L[i + j * ldl];
    }
}

template <typename T>
void potrf(T* A, int64_t lda, int n, int* err, int64_t* err_col, int64_t col_offset, cudaStream_t s) {
    ProfScope prof_("potrf", s);
    const size_t sm = (size_t)n * (n + 1) * sizeof(T);
    if (sm > 227 * 1024) throw Error(OMG_ERR_INVALID, "diagonal block too large for shared memory");
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(potrf_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        attr = true;
    }
    potrf_kernel<T><<<1, 512, sm, s>>>(A, lda, n, err, err_col, col_offset);
    check("potrf");
}
template void potrf<double>(double*, int64_t, int, int*, int64_t*, int64_t, cudaStream_t);
template void potrf<float>(float*, int64_t, int, int*, int64_t*, int64_t, cudaStream_t);

// ---------------------------------------------------------------------------
// Triangular solves with a diagonal block L (n x n lower, staged in shared
// memory).  Panel form (rows independent):  W = P L^-T  for P (m x n).
// Column form (columns independent):       B <- L^-1 B  or  L^-T B.
// Each row / column is one warp: the substitution runs serially over the
// block, the inner products across the 32 lanes.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) trsm_rows_kernel(int64_t m, int n, const T* __restrict__ L, int64_t ldl,
                                                        T* P, int64_t ldp) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T* sL = reinterpret_cast<T*>(smraw);          // n x n (row-major copy: sL[j*n + l] = L[j][l])
    T* sx = sL + n * n;                           // 8 warps x n
    for (int e = threadIdx.x; e < n * n; e += 256) {   // coalesced read down the columns of L
        const int j = e % n, l = e / n;
        sL[j * n + l] = (l <= j) ? L[j + l * ldl] : T(0);
    }
    __syncthreads();
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    T* x = sx + warp * n;
    for (int64_t row = (int64_t)blockIdx.x * 8 + warp; row < m; row += (int64_t)gridDim.x * 8) {
        for (int l = lane; l < n; l += 32) x[l] = P[row + (int64_t)l * ldp];
        __syncwarp();
        // x L^T = p  <=>  L x^T = p^T : forward substitution over j
        for (int j = 0; j < n; ++j) {
            T acc = T(0);
            for (int l = lane; l < j; l += 32) acc += x[l] * sL[j * n + l];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) x[j] = (x[j] - acc) / sL[j * n + j];
            __syncwarp();
        }
        for (int l = lane; l < n; l += 32) P[row + (int64_t)l * ldp] = x[l];
        __syncwarp();
    }
}

template <typename T>
__global__ void __launch_bounds__(256) trsm_cols_kernel(int64_t nrhs, int n, const T* __restrict__ L, int64_t ldl,
                                                        const T* __restrict__ Lr, int trans, T* B, int64_t ldb) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T* sL = reinterpret_cast<T*>(smraw);   // n x n, sL[j*n + l] = (trans ? L[l][j] : L[j][l]) for the used part
    T* sx = sL + n * n;
    for (int e = threadIdx.x; e < n * n; e += 256) {   // coalesced: r runs down column c of L
        const int r = e % n, c = e / n;
        const T v = (r >= c) ? (Lr ? L[r + c * ldl] + Lr[r + c * ldl] : L[r + c * ldl]) : T(0);
        if (trans)
            sL[c * n + r] = v;   // (L^T)[c][r]
        else
            sL[r * n + c] = v;   // L[r][c]
    }
    __syncthreads();
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    T* x = sx + warp * n;
    for (int64_t col = (int64_t)blockIdx.x * 8 + warp; col < nrhs; col += (int64_t)gridDim.x * 8) {
        T* b = B + col * ldb;
        for (int l = lane; l < n; l += 32) x[l] = b[l];
        __syncwarp();
        if (!trans) {   // L x = b, forward
            for (int j = 0; j < n; ++j) {
                T acc = T(0);
                for (int l = lane; l < j; l += 32) acc += sL[j * n + l] * x[l];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (lane == 0) x[j] = (x[j] - acc) / sL[j * n + j];
                __syncwarp();
            }
        } else {        // L^T x = b, backward: row j of L^T is column j of L
            for (int j = n - 1; j >= 0; --j) {
                T acc = T(0);
                for (int l = j + 1 + lane; l < n; l += 32) acc += sL[j * n + l] * x[l];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (lane == 0) x[j] = (x[j] - acc) / sL[j * n + j];
                __syncwarp();
            }
        }
        for (int l = lane; l < n; l += 32) b[l] = x[l];
        __syncwarp();
    }
}

template <typename T>
static void set_max_smem(const void* f) {
    cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}

template <typename T>
void trsm_rows(int64_t m, int n, const T* L, int64_t ldl, T* P, int64_t ldp, cudaStream_t s) {
    if (m <= 0) return;
    ProfScope prof_("trsm_rows", s);
    static bool attr = false;
    if (!attr) {
        set_max_smem<T>((const void*)trsm_rows_kernel<T>);
        attr = true;
    }
    const size_t sm = ((size_t)n * n + 8 * (size_t)n) * sizeof(T);
    const unsigned grid = (unsigned)std::min<int64_t>((m + 7) / 8, 152 * 8);
    trsm_rows_kernel<T><<<grid, 256, sm, s>>>(m, n, L, ldl, P, ldp);
    check("trsm_rows");
}
template <typename T>
void trsm_cols(int64_t nrhs, int n, const T* L, int64_t ldl, bool trans, T* B, int64_t ldb, cudaStream_t s,
               const T* Lr) {
    if (nrhs <= 0) return;
    ProfScope prof_("trsm_cols", s);
    static bool attr = false;
    if (!attr) {
        set_max_smem<T>((const void*)trsm_cols_kernel<T>);
        attr = true;
    }
    const size_t sm = ((size_t)n * n + 8 * (size_t)n) * sizeof(T);
    const unsigned grid = (unsigned)std::min<int64_t>((nrhs + 7) / 8, 152 * 8);
    trsm_cols_kernel<T><<<grid, 256, sm, s>>>(nrhs, n, L, ldl, Lr, trans ? 1 : 0, B, ldb);
    check("trsm_cols");
}
template void trsm_rows<double>(int64_t, int, const double*, int64_t, double*, int64_t, cudaStream_t);
template void trsm_rows<float>(int64_t, int, const float*, int64_t, float*, int64_t, cudaStream_t);
template void trsm_cols<double>(int64_t, int, const double*, int64_t, bool, double*, int64_t, cudaStream_t,
                                const double*);
template void trsm_cols<float>(int64_t, int, const float*, int64_t, bool, float*, int64_t, cudaStream_t, const float*);

// Max-norm of each column of an m x n FP32 matrix scaled by colscale, and of
// an FP64 matrix: one CTA per column (for the refinement stopping test).
__global__ void col_amax_kernel(int64_t m, const double* __restrict__ A, int64_t lda, double* out) {
    __shared__ double red[256];
    const int64_t j = blockIdx.x;
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) s = fmax(s, fabs(A[i + j * lda]));
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[j] = red[0];
}
// 2-norms of the columns of an FP32 matrix times a per-column scale.
__global__ void col_norms_f32_kernel(int64_t m, const float* __restrict__ A, int64_t lda,
                                     const double* __restrict__ scale, double* out) {
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
    if (threadIdx.x == 0) out[j] = sqrt(red[0]) * (scale ? scale[j] : 1.0);
}
void col_norms_f32(int64_t m, int64_t n, const float* A, int64_t lda, const double* scale, double* out,
                   cudaStream_t s) {
    if (n <= 0) return;
    ProfScope prof_("col_norms", s);
    col_norms_f32_kernel<<<(unsigned)n, 256, 0, s>>>(m, A, lda, scale, out);
    check("col_norms_f32");
}

// out[0] = max_j num[j] / den[j] over columns with den[j] > 0 (a NaN ratio
// gives +inf, so a broken column can never pass a tolerance test).
__global__ void ratio_max_kernel(int64_t n, const double* __restrict__ num, const double* __restrict__ den,
                                 double* out) {
    __shared__ double red[256];
    double m = 0.0;
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        if (den[j] > 0.0) {
            const double r = num[j] / den[j];
            m = (r != r) ? INFINITY : fmax(m, r);
        } else if (den[j] != den[j]) {
            m = INFINITY;
        }
    }
    red[threadIdx.x] = m;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = red[0];
}
void ratio_max(int64_t n, const double* num, const double* den, double* out, cudaStream_t s) {
    ratio_max_kernel<<<1, 256, 0, s>>>(n, num, den, out);
    check("ratio_max");
}

void col_amax(int64_t m, int64_t n, const double* A, int64_t lda, double* out, cudaStream_t s) {
    if (n <= 0) return;
    ProfScope prof_("col_amax", s);
    col_amax_kernel<<<(unsigned)n, 256, 0, s>>>(m, A, lda, out);
    check("col_amax");
}

// ---------------------------------------------------------------------------
// Diagonal block of the FP32 factorization: Cholesky of the n x n (n <= 128)
// block A11 and the inverse of its factor, in one CTA of 512 threads, blocked
// by 32 columns (4 block steps J):
//   1. warp 0 factors the 32 x 32 diagonal block in registers (lane i holds
//      row i, shifted so the current column is in a fixed register; the
//      unscaled column j is broadcast through shared memory while the pivot's
//      reciprocal square root is formed, so the update a_ik -= a_ij a_kj / a_jj
//      waits for one multiply after the broadcast), no CTA barrier inside;
//   2. warp 0 inverts that block (lane c solves column c of X_JJ) while the
//      threads of warps 1-3 solve one panel row each, L_rJ = A_rJ L_JJ^-T, by
//      forward substitution (rows below the block);
//   3. the rank-32 update of the trailing lower triangle in 4 x 4 register
//      tiles, reading the panel from a k-major copy;
// the off-diagonal blocks of the inverse, X_JK = -X_JJ sum_{M=K}^{J-1} L_JM
// X_MK, are computed block row by block row inside the same loop.  With a
// look-ahead, warp 0 factors block J+1 as soon as that block alone is
// updated: warp 1's panel rows (those of block J+1) are handed to warps 4-15,
// which update block J+1 beside the other panel rows and X_JJ; the rest of the
// trailing update, block row J of the inverse and the sums of block row J+1
// then run while warp 0 factors block J+1 (two named barriers), on the 12
// warps outside warp 0's scheduler partition (sharing it, the factorization's
// serial steps lost most of their issue slots and nothing was gained).
// The block lives in shared memory (row-major, padded); columns past n act as
// the identity.

// Outputs: L11 over A11 (lower; left out when store_l is false: the
// factorization's solves use only the inverse), Linv as TF32 head/remainder
// K-major rows (128 x 128 each, zero padded) for the tensor-core panel solve
// L21 = A21 Linv^T, and, when Linv is not null, Linv column-major (ldi = 128,
// zero above the diagonal and beyond n).  The factorization leaves Linv null
// and transposes all the blocks' splits at its end (linv_from_split): the
// chain of diagonal blocks then stores 128 KB per block instead of 192 KB.
// A pivot that is not a positive normal FP32 number is reported as
// OMG_ERR_NOT_DEFINITE at its column (and replaced by 1 so the kernel ends).
// ---------------------------------------------------------------------------
constexpr int PI_NB = 128, PI_LD = 129, PI_THREADS = 512, PI_BS = 32, PI_TLD = 33;
constexpr size_t PI_SMEM =
    ((size_t)2 * PI_NB * PI_LD + (size_t)PI_BS * PI_NB + 3 * PI_BS * PI_TLD + PI_NB + 2 * PI_BS) * sizeof(float);

// Block row J of the inverse X = L^-1 (32-row blocks), one 4 x 4 tile t of
// the J x 64 tiles of its blocks K < J: T_JK = sum_{M=K}^{J-1} L_JM X_MK (the
// rows of L in sA, of X in sX, T into sT), then X_JK = -X_JJ T_JK.
__device__ __forceinline__ void pi_inv_rowblock_t(const float* sA, const float* sX, float* sT, int J, int t) {
    const int K = t / 64, ti = (t % 64) / 8, tj = t % 8;
    const int r0 = PI_BS * J + 4 * ti, c0 = PI_BS * K + 4 * tj;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int k = PI_BS * K; k < PI_BS * J; ++k) {
        float av[4], bv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) av[i] = sA[(r0 + i) * PI_LD + k];
#pragma unroll
        for (int j = 0; j < 4; ++j) bv[j] = sX[k * PI_LD + c0 + j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    float* T = sT + K * PI_BS * PI_TLD;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) T[(4 * ti + i) * PI_TLD + 4 * tj + j] = acc[i][j];
}

__device__ __forceinline__ void pi_inv_rowblock_x(float* sX, const float* sT, int J, int t) {
    const int K = t / 64, ti = (t % 64) / 8, tj = t % 8;
    const int r0 = PI_BS * J + 4 * ti, c0 = PI_BS * K + 4 * tj;
    const float* T = sT + K * PI_BS * PI_TLD;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int k = 0; k < PI_BS; ++k) {
        float av[4], bv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) av[i] = sX[(r0 + i) * PI_LD + PI_BS * J + k];
#pragma unroll
        for (int j = 0; j < 4; ++j) bv[j] = T[k * PI_TLD + 4 * tj + j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) sX[(r0 + i) * PI_LD + c0 + j] = -acc[i][j];
}

// One 4 x 4 tile t (lower triangle, row-major tile order) of the rank-32 update of the trailing lower
// triangle from row and column b by the panel in sP (k-major): A_rc -= sum_k P_rk P_ck, r >= c.
__device__ __forceinline__ void pi_trailing_tile(float* sA, const float* sP, int b, int t) {
    int ti = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);
    while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
    while (ti * (ti + 1) / 2 > t) --ti;
    const int tj = t - ti * (ti + 1) / 2;
    const int r0 = b + 4 * ti, c0 = b + 4 * tj;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
#pragma unroll 8
    for (int k = 0; k < PI_BS; ++k) {
        const float4 a = *reinterpret_cast<const float4*>(sP + k * PI_NB + r0);
        const float4 c = *reinterpret_cast<const float4*>(sP + k * PI_NB + c0);
        const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (c0 + j <= r0 + i) sA[(r0 + i) * PI_LD + c0 + j] -= acc[i][j];
}

__global__ void __launch_bounds__(PI_THREADS, 1) potrf_inv_kernel(float* A, int64_t lda, int n, int* err,
                                                               int64_t* err_col, int64_t col_offset, float* Linv,
                                                               float* Bh, float* Bl, int store_l) {
    extern __shared__ __align__(16) unsigned char smraw[];
    float* sA = reinterpret_cast<float*>(smraw);   // 128 x PI_LD row-major: A, then L
    float* sX = sA + PI_NB * PI_LD;                 // 128 x PI_LD row-major: X = L^-1
    float* sP = sX + PI_NB * PI_LD;                 // 32 x 128: panel column block, k-major (sP[k * 128 + r])
    float* sT = sP + PI_BS * PI_NB;                 // 3 x 32 x PI_TLD: T blocks of the inverse
    float* sInv = sT + 3 * PI_BS * PI_TLD;          // 1 / L[j][j]
    float* sCol = sInv + PI_NB;                     // 2 x 32: column broadcast of the diagonal factor
    const unsigned FULL = 0xffffffffu;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    asm volatile("griddepcontrol.launch_dependents;");
    asm volatile("griddepcontrol.wait;" ::: "memory");   // the block's last update (no-op without PDL)
    // the lower triangle by 4-byte asynchronous copies (a thread's 32 in flight at once, no registers
    // held), coalesced down the columns of A, in two groups: the first column block (all the first
    // diagonal block needs) and the rest, which lands while warp 0 factors that block; identity beyond
    // n, zero above the diagonal
#pragma unroll 1
    for (int i = 0; i < PI_NB * PI_NB / PI_THREADS; ++i) {
        const int e = tid + i * PI_THREADS;
        const int r = e % PI_NB, c = e / PI_NB;
        float* dst = sA + r * PI_LD + c;
        if (r >= c && r < n) {   // c <= r < n
            const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(A + r + (int64_t)c * lda)
                         : "memory");
        } else {
            *dst = (r == c) ? 1.f : 0.f;
        }
        sX[r * PI_LD + c] = 0.f;
        if (i == PI_BS * PI_NB / PI_THREADS - 1) asm volatile("cp.async.commit_group;" ::: "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 1;" ::: "memory");   // this thread's copies of the first column block
    __syncthreads();
    // Look-ahead: each diagonal block is factored as soon as its own update is complete.
    //   phase 1 (J): warp 0 factors diagonal block J; the warps of the other scheduler partitions apply
    //                the rest of panel J-1's trailing update (rows past block J), finish block row J-1 of
    //                the inverse and form the sums T_JK of block row J (named barrier 1 between the two)
    //   phase 2 (J): warp 0 inverts L_JJ; warps 1-3 solve the panel rows; warp 1's rows (those of block
    //                J+1) go first to warps 5 and 6, which update diagonal block J+1 by them (named
    //                barrier 2)
    for (int J = 0; J < 4; ++J) {
        const int j0 = J * PI_BS;
        if (warp == 0) {   // ---- 1. Cholesky of the diagonal block
            // lane i holds row i, shifted left by one column per step so that the current column
            // sits in r[0]; the unscaled column j (a_(j+m)j at cb[m], the pivot at cb[0]) is broadcast
            // through shared memory and read back as 8 aligned float4 (static offsets) while the
            // pivot comes by shuffle and its reciprocal square root is formed
            float r[PI_BS];
#pragma unroll
            for (int m = 0; m < PI_BS; ++m) r[m] = (m <= lane) ? sA[(j0 + lane) * PI_LD + j0 + m] : 0.f;
            unsigned badmask = 0u;   // a bit per pivot that is not a positive normal number
#pragma unroll 1
            for (int j = 0; j < PI_BS; ++j) {
                const float u = r[0];   // a_(lane)j after the updates by the columns before j
                const float ub = lane > j ? u : 0.f;   // rows j and above are final: no update
                float* cb = sCol + (j & 1) * PI_BS;
                if (lane >= j) cb[lane - j] = u;
                float d = __shfl_sync(FULL, u, j);
                __syncwarp();
                // branch-free (a branch here doubled the step's latency); NaN fails the test too
                const bool ok = d >= 1.17549435e-38f;
                badmask |= ok ? 0u : (1u << j);
                d = ok ? d : 1.f;
                float inv;   // 1 / sqrt(d), the PTX approximation (relative error below 2^-22)
                asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(d));
                const float sc = ub * (inv * inv);   // l_ij / l_jj
                sA[(j0 + lane) * PI_LD + j0 + j] = (lane == j) ? d * inv : (lane > j ? u * inv : 0.f);
                if (lane == j) sInv[j0 + j] = inv;
                // a[i][j + m] -= (a_ij / a_jj) a_(j+m)j; slots past the block read stale values and are
                // never pivots
#pragma unroll
                for (int q = 0; q < PI_BS / 4; ++q) {
                    const float4 c4 = reinterpret_cast<const float4*>(cb)[q];
                    const float cv[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        const int m = 4 * q + t;
                        if (m >= 1) r[m - 1] = fmaf(-sc, cv[t], r[m]);
                    }
                }
                r[PI_BS - 1] = 0.f;
            }
            if (badmask && lane == 0 && atomicCAS(err, 0, -3 /* OMG_ERR_NOT_DEFINITE */) == 0)
                *err_col = col_offset + j0 + (__ffs((int)badmask) - 1);
            if (J == 0) asm volatile("cp.async.wait_group 0;" ::: "memory");
        } else if (J == 0) {
            asm volatile("cp.async.wait_group 0;" ::: "memory");   // the rest of the block
        } else if (warp & 3) {
            // helpers: the 12 warps outside warp 0's scheduler partition (warp w issues on partition w % 4),
            // so the factorization's latency-bound steps keep their issue slots; warps 4, 8, 12 wait
            const int ht = (warp - 1 - (warp >> 2)) * 32 + lane, nh = 12 * 32;
            // ---- 3. the rest of panel J-1's trailing update: 4 x 4 tiles of its lower trailing triangle
            // (from row and column j0) past the first 8 tile rows, which are diagonal block J (updated in
            // phase 2 of J-1)
            const int tm = (PI_NB - j0) / 4, ntiles = tm * (tm + 1) / 2;
            for (int t = 36 + ht; t < ntiles; t += nh) pi_trailing_tile(sA, sP, j0, t);
            if (J > 1)   // ---- 3'. X_(J-1)K = -X_(J-1)(J-1) T_(J-1)K, K < J-1
                for (int t = ht; t < (J - 1) * 64; t += nh) pi_inv_rowblock_x(sX, sT, J - 1, t);
            asm volatile("bar.sync 1, %0;" ::"n"(12 * 32) : "memory");   // the helpers
            // ---- 1'. T_JK = sum_{M=K}^{J-1} L_JM X_MK for K < J (needs block row J-1 of the inverse)
            for (int t = ht; t < J * 64; t += nh) pi_inv_rowblock_t(sA, sX, sT, J, t);
        }
        __syncthreads();
        const int below = PI_NB - j0 - PI_BS;
        if (warp == 0) {   // ---- 2a. X_JJ = L_JJ^-1, column `lane`
            float x[PI_BS];
#pragma unroll
            for (int r = 0; r < PI_BS; ++r) {
                const float* Lr = sA + (j0 + r) * PI_LD + j0;
                float acc0 = (r == lane) ? 1.f : 0.f, acc1 = 0.f;
#pragma unroll
                for (int k = 0; k < r; ++k) {
                    if (k & 1)
                        acc1 = fmaf(-Lr[k], x[k], acc1);
                    else
                        acc0 = fmaf(-Lr[k], x[k], acc0);
                }
                x[r] = (acc0 + acc1) * sInv[j0 + r];
            }
#pragma unroll
            for (int r = 0; r < PI_BS; ++r) sX[(j0 + r) * PI_LD + j0 + lane] = x[r];
        } else if (warp < 4) {
            if (tid - 32 < below) {   // ---- 2b. one panel row: L_rJ L_JJ^T = A_rJ
                const int r = j0 + PI_BS + (tid - 32);
                float l[PI_BS];
#pragma unroll
                for (int j = 0; j < PI_BS; ++j) {
                    const float* Lj = sA + (j0 + j) * PI_LD + j0;
                    float acc0 = sA[r * PI_LD + j0 + j], acc1 = 0.f;
#pragma unroll
                    for (int k = 0; k < j; ++k) {
                        if (k & 1)
                            acc1 = fmaf(-l[k], Lj[k], acc1);
                        else
                            acc0 = fmaf(-l[k], Lj[k], acc0);
                    }
                    l[j] = (acc0 + acc1) * sInv[j0 + j];
                }
#pragma unroll
                for (int j = 0; j < PI_BS; ++j) {
                    sA[r * PI_LD + j0 + j] = l[j];
                    sP[j * PI_NB + r] = l[j];
                }
            }
            if (warp == 1 && below > 0) {   // the rows of diagonal block J+1 are in
                __threadfence_block();
                asm volatile("bar.arrive 2, %0;" ::"n"(3 * 32) : "memory");   // warps 1, 5, 6
            }
        } else if ((warp == 5 || warp == 6) && below > 0) {
            // ---- 3. diagonal block J+1 by panel J: the first 36 tiles of its trailing triangle (on
            // partitions 1 and 2, beside warp 0's inverse of L_JJ)
            asm volatile("bar.sync 2, %0;" ::"n"(3 * 32) : "memory");
            for (int t = (warp - 5) * 32 + lane; t < 36; t += 64) pi_trailing_tile(sA, sP, j0 + PI_BS, t);
        }
        __syncthreads();
    }
    for (int t = tid; t < 3 * 64; t += PI_THREADS) pi_inv_rowblock_x(sX, sT, 3, t);   // X_3K = -X_33 T_3K
    __syncthreads();
    if (store_l) {
        for (int e = tid; e < PI_NB * PI_NB; e += PI_THREADS) {   // no division by the runtime size
            const int r = e % PI_NB, c = e / PI_NB;
            if (r >= c && r < n) A[r + (int64_t)c * lda] = sA[r * PI_LD + c];
        }
    }
    // one element per thread and step, consecutive lanes on consecutive (bank-distinct) words of the
    // padded rows and columns of X, 128-byte coalesced stores
#pragma unroll 4
    for (int e = tid; e < PI_NB * PI_NB; e += PI_THREADS) {   // K-major rows: B[rr][cc] = Linv[rr][cc]
        const int rr = e / PI_NB, cc = e % PI_NB;
        const float w = (rr < n && cc < n) ? sX[rr * PI_LD + cc] : 0.f;
        const float h = __uint_as_float(__float_as_uint(w) & 0xFFFFE000u);
        Bh[e] = h;
        Bl[e] = w - h;
    }
    if (Linv) {
        for (int e = tid; e < PI_NB * PI_NB; e += PI_THREADS) {   // column-major Linv
            const int r = e % PI_NB, c = e / PI_NB;
            Linv[e] = (r < n && c < n) ? sX[r * PI_LD + c] : 0.f;
        }
    }
}

void potrf_inv(float* A, int64_t lda, int n, int* err, int64_t* err_col, int64_t col_offset, float* Linv, float* Bh,
               float* Bl, cudaStream_t s, bool store_l, bool pdl) {
    if (n <= 0 || n > PI_NB) throw Error(OMG_ERR_INVALID, "diagonal block must have 1..128 columns");
    ProfScope prof_("potrf_inv", s);
    const size_t sm = PI_SMEM;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(potrf_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        attr = true;
    }
    launch_maybe_pdl(pdl, potrf_inv_kernel, 1, PI_THREADS, sm, s, A, lda, n, err, err_col, col_offset, Linv, Bh, Bl,
                     store_l ? 1 : 0);
    check("potrf_inv");
}

// The diagonal-block inverses from their K-major splits (block b: heads at
// B + 2 b 128^2, remainders 128^2 further, row-major 128 x 128): Linv
// column-major (ld 128, block b at b 128^2) and its split as stored, LCh / LCl
// (the same layout).  head + remainder is exactly the FP32 value, so Linv is
// bit-identical to the inverse the diagonal-block kernel computed.  One 32 x 32
// tile per CTA, transposed through shared memory.
__global__ void linv_from_split_kernel(const float* __restrict__ B, float* __restrict__ Linv, float* __restrict__ LCh,
                                       float* __restrict__ LCl) {
    __shared__ float th[32][33], tl[32][33];
    const int64_t blk = (int64_t)blockIdx.x * PI_NB * PI_NB;
    const float* Bh = B + 2 * blk;
    const float* Bl = Bh + PI_NB * PI_NB;
    const int r0 = 32 * blockIdx.y, c0 = 32 * blockIdx.z, x = threadIdx.x;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {   // rows r0 + y, columns c0 + x of the inverse
        th[y][x] = Bh[(r0 + y) * PI_NB + c0 + x];
        tl[y][x] = Bl[(r0 + y) * PI_NB + c0 + x];
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {   // column c0 + y, rows r0 + x
        const float h = th[x][y], l = tl[x][y];
        const int64_t o = blk + (int64_t)(c0 + y) * PI_NB + r0 + x;
        Linv[o] = h + l;
        LCh[o] = h;
        LCl[o] = l;
    }
}

void linv_from_split(int64_t nblocks, const float* B, float* Linv, float* LCh, float* LCl, cudaStream_t s) {
    if (nblocks <= 0) return;
    ProfScope prof_("linv_from_split", s);
    linv_from_split_kernel<<<dim3((unsigned)nblocks, PI_NB / 32, PI_NB / 32), dim3(32, 8), 0, s>>>(B, Linv, LCh, LCl);
    check("linv_from_split");
}

// Symmetric update of an n x n (n <= 128) diagonal block by up to two panels
// of the factorization, A11 -= P0 P0^T + P1 P1^T, lower triangle, FP32 FMA in
// a fixed order (panel 0, then panel 1, k ascending).  Each panel is given as
// the TF32 head and remainder rows of its K-major split (n rows of 128
// values; head + remainder = the FP32 panel).  One CTA per lower 32 x 32
// block (10), 256 threads, 2 x 2 outputs each; both 32-row slices of a panel
// are staged in shared memory (row-major, padded: the threads of a warp read
// 16 different rows of one column, conflict free).
constexpr int DU_LD = 129;
__global__ void __launch_bounds__(256) diag_update_kernel(float* A, int64_t lda, int n, const float* __restrict__ P0h,
                                                         const float* __restrict__ P0l,
                                                         const float* __restrict__ P1h,
                                                         const float* __restrict__ P1l) {
    __shared__ float sI[32 * DU_LD], sJ[32 * DU_LD];
    asm volatile("griddepcontrol.launch_dependents;");
    asm volatile("griddepcontrol.wait;" ::: "memory");   // the panel rows (no-op without PDL)
    int I = 0, t = blockIdx.x;   // lower block (I, J) number t = I (I + 1) / 2 + J
    while (t > I) t -= ++I;
    const int J = t, tid = threadIdx.x;
    const int r0 = 32 * I + 2 * (tid >> 4), c0 = 32 * J + 2 * (tid & 15);
    float acc[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    for (int p = 0; p < 2; ++p) {
        const float* Ph = p ? P1h : P0h;
        const float* Pl = p ? P1l : P0l;
        if (!Ph) break;
        if (p) __syncthreads();
#pragma unroll 4
        for (int e = tid; e < 2 * 32 * 32; e += 256) {   // (slice, row, 4 values): float4 reads along the rows
            const int q = e & 31, row = (e >> 5) & 31, sl = e >> 10;
            const int gr = 32 * (sl ? J : I) + row;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (gr < n) {
                const float4 h = *reinterpret_cast<const float4*>(Ph + (int64_t)gr * 128 + 4 * q);
                const float4 l = *reinterpret_cast<const float4*>(Pl + (int64_t)gr * 128 + 4 * q);
                v = make_float4(h.x + l.x, h.y + l.y, h.z + l.z, h.w + l.w);
            }
            float* d = (sl ? sJ : sI) + row * DU_LD + 4 * q;
            d[0] = v.x;
            d[1] = v.y;
            d[2] = v.z;
            d[3] = v.w;
        }
        __syncthreads();
        const float* a0 = sI + (r0 - 32 * I) * DU_LD;
        const float* b0 = sJ + (c0 - 32 * J) * DU_LD;
#pragma unroll 8
        for (int k = 0; k < 128; ++k) {
            const float x0 = a0[k], x1 = a0[DU_LD + k], y0 = b0[k], y1 = b0[DU_LD + k];
            acc[0][0] = fmaf(x0, y0, acc[0][0]);
            acc[0][1] = fmaf(x0, y1, acc[0][1]);
            acc[1][0] = fmaf(x1, y0, acc[1][0]);
            acc[1][1] = fmaf(x1, y1, acc[1][1]);
        }
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int r = r0 + i, c = c0 + j;
            if (r >= c && r < n) A[r + (int64_t)c * lda] -= acc[i][j];
        }
}

void diag_update(float* A, int64_t lda, int n, const float* P0h, const float* P0l, const float* P1h, const float* P1l,
                 cudaStream_t s, bool pdl) {
    if (n <= 0 || n > 128) throw Error(OMG_ERR_INVALID, "diagonal block must have 1..128 columns");
    for (const float* q : {P0h, P0l, P1h, P1l})
        if (reinterpret_cast<uintptr_t>(q) % 16) throw Error(OMG_ERR_INVALID, "panel rows not 16-byte aligned");
    if (!P0h || !P0l || !P1h != !P1l) throw Error(OMG_ERR_INVALID, "panel update needs heads and remainders");
    ProfScope prof_("diag_update", s);
    const int nb32 = (n + 31) / 32;
    launch_maybe_pdl(pdl, diag_update_kernel, nb32 * (nb32 + 1) / 2, 256, 0, s, A, lda, n, P0h, P0l, P1h, P1l);
    check("diag_update");
}

// B <- blockdiag(op(Linv_b)) B over all diagonal blocks at once, op =
// transpose if `trans`: block b covers rows b*128 .. b*128 + n_b - 1 (n_b =
// 128 but for the last block, n_last) of the N x ncol matrix B (ldb); Linv_b
// are the column-major 128 x 128 inverses, zero outside n_b x n_b.  Grid
// (column groups, blocks): each CTA stages op(Linv_b) once in shared memory
// (column-major, sM[i + l*ldm]) and then takes 32 columns per pass; each
// thread accumulates a 4 x 4 tile (rows 4*tr.., columns 4*tc..) from 128-bit
// shared loads (one operand read per four products).
constexpr int AB_THREADS = 256, AB_COLS = 32, AB_NB = 128, AB_LDM = AB_NB + 4;
constexpr size_t AB_SMEM = (size_t)(AB_NB + AB_COLS) * AB_LDM * sizeof(float);

__global__ void __launch_bounds__(AB_THREADS) apply_inv_blocks_kernel(int nblocks, int n_last, int64_t ncol,
                                                                      const float* __restrict__ Li, int trans,
                                                                      float* B, int64_t ldb) {
    extern __shared__ __align__(16) unsigned char smraw[];
    float* sM = reinterpret_cast<float*>(smraw);   // sM[i + l*AB_LDM] = op(Linv_b)[i][l]
    float* sB = sM + AB_NB * AB_LDM;               // sB[c*AB_LDM + l] = B(b*128 + l, j0 + c)
    const int blk = blockIdx.y;
    const int n = blk == nblocks - 1 ? n_last : AB_NB;
    const float* L = Li + (int64_t)blk * AB_NB * AB_NB;
    float* Bb = B + (int64_t)blk * AB_NB;
    for (int e = threadIdx.x; e < AB_NB * AB_NB; e += AB_THREADS) {
        const int r = e % AB_NB, c = e / AB_NB;   // coalesced read of column-major Linv
        const float v = L[r + c * AB_NB];
        if (trans)
            sM[c + r * AB_LDM] = v;
        else
            sM[r + c * AB_LDM] = v;
    }
    const int tr = threadIdx.x % 32, tc = threadIdx.x / 32;   // tc is uniform in a warp: broadcast reads of sB
    const int64_t npass = (ncol + AB_COLS - 1) / AB_COLS;
    for (int64_t p = blockIdx.x; p < npass; p += gridDim.x) {
        const int64_t j0 = p * AB_COLS;
        __syncthreads();   // the staged block (first pass) / the previous pass's reads of sB
        for (int e = threadIdx.x; e < AB_NB * AB_COLS; e += AB_THREADS) {
            const int l = e % AB_NB, c = e / AB_NB;
            sB[c * AB_LDM + l] = (l < n && j0 + c < ncol) ? Bb[l + (j0 + c) * ldb] : 0.f;
        }
        __syncthreads();
        float acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[i][c] = 0.f;
#pragma unroll 2
        for (int l = 0; l < AB_NB; l += 4) {
            float4 a[4], bv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) a[u] = *reinterpret_cast<const float4*>(sM + 4 * tr + (l + u) * AB_LDM);
#pragma unroll
            for (int c = 0; c < 4; ++c) bv[c] = *reinterpret_cast<const float4*>(sB + (4 * tc + c) * AB_LDM + l);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const float b4[4] = {bv[c].x, bv[c].y, bv[c].z, bv[c].w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    acc[0][c] = fmaf(a[u].x, b4[u], acc[0][c]);
                    acc[1][c] = fmaf(a[u].y, b4[u], acc[1][c]);
                    acc[2][c] = fmaf(a[u].z, b4[u], acc[2][c]);
                    acc[3][c] = fmaf(a[u].w, b4[u], acc[3][c]);
                }
            }
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int64_t j = j0 + 4 * tc + c;
            if (j >= ncol) continue;
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (4 * tr + i < n) Bb[4 * tr + i + j * ldb] = acc[i][c];
        }
    }
}

void apply_inv_blocks(int64_t nblocks, int nb, int n_last, int64_t ncol, const float* Li, bool trans, float* B,
                      int64_t ldb, cudaStream_t s) {
    if (nblocks <= 0 || ncol <= 0) return;
    if (nb != AB_NB || n_last < 1 || n_last > nb || nblocks > 65535)
        throw Error(OMG_ERR_INVALID, "apply_inv_blocks: unsupported block layout");
    ProfScope prof_("apply_inv", s);
    static bool attr = false;
    static int n_sm = 0;
    if (!attr) {
        cudaFuncSetAttribute(apply_inv_blocks_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)AB_SMEM);
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
        if (n_sm <= 0) n_sm = 1;
        attr = true;
    }
    // about two CTAs per SM in all: fewer passes per CTA than stagings of Linv_b
    const int64_t npass = (ncol + AB_COLS - 1) / AB_COLS;
    const int64_t groups = std::max<int64_t>(1, std::min<int64_t>(npass, (2 * n_sm + nblocks - 1) / nblocks));
    dim3 grid((unsigned)groups, (unsigned)nblocks);
    apply_inv_blocks_kernel<<<grid, AB_THREADS, AB_SMEM, s>>>((int)nblocks, n_last, ncol, Li, trans ? 1 : 0, B, ldb);
    check("apply_inv_blocks");
}

}  // namespace omg

// Test hook (not part of the public header): factor and invert one diagonal
// block (device pointers), after the update by the panels P0, P1 when given
// (diag_update: head / remainder rows, 128 values each; null for none).  With
// reps > 1 the call is then repeated on scratch copies and the mean time of
// the launches (microseconds, CUDA events on the default stream) is returned
// through *us.
extern "C" int omg_internal_potrf_inv(int n, float* A, int64_t lda, float* Linv, float* Bh, float* Bl, int* err,
                                      int reps, float* us, const float* P0h, const float* P0l, const float* P1h,
                                      const float* P1l) {
    int64_t* col = nullptr;
    float* scratch = nullptr;
    int* err2 = nullptr;
    int rc = 0;
    try {
        if (cudaMalloc(&col, sizeof(int64_t)) != cudaSuccess || cudaMalloc(&err2, sizeof(int)) != cudaSuccess ||
            cudaMalloc(&scratch, sizeof(float) * 4 * 128 * 128) != cudaSuccess)
            throw omg::Error(OMG_ERR_NOMEM, "test hook allocation");
        cudaMemset(err2, 0, sizeof(int));
        if (reps > 1) {   // scratch copy of the input block first (the first call overwrites A)
            cudaMemcpy2D(scratch, 128 * sizeof(float), A, lda * sizeof(float), n * sizeof(float), n,
                         cudaMemcpyDeviceToDevice);
        }
        if (P0h) omg::diag_update(A, lda, n, P0h, P0l, P1h, P1l, 0, false);
        omg::potrf_inv(A, lda, n, err, col, 0, Linv, Bh, Bl, 0, true, false);
        if (reps > 1) {
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            float* s1 = scratch + 128 * 128;
            cudaEventRecord(e0, 0);
            for (int r = 1; r < reps; ++r) {   // same work on a scratch block (values no longer matter)
                if (P0h) omg::diag_update(scratch, 128, n, P0h, P0l, P1h, P1l, 0, false);
                omg::potrf_inv(scratch, 128, n, err2, col, 0, s1, s1 + 128 * 128, s1 + 2 * 128 * 128, 0, false,
                               false);
            }
            cudaEventRecord(e1, 0);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (us) *us = 1000.f * ms / (float)(reps - 1);
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
        }
        rc = cudaDeviceSynchronize() == cudaSuccess ? 0 : -2;
    } catch (const omg::Error& e) {
        rc = e.code;
    }
    cudaFree(col);
    cudaFree(err2);
    cudaFree(scratch);
    return rc;
}

namespace omg {

// ---------------------------------------------------------------------------
// Pipe peaks for the rooflines of the CUDA-core kernels (no measured FP32 /
// FP64 figure comes with the machine): every thread runs 8 independent FMA
// chains for `iters` steps, a grid of 8 CTAs of 256 threads per SM.  Returns
// FMA instructions (per lane) per second, timed with CUDA events.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) fma_peak_kernel(int iters, T a, T b, T* out) {
    T x[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = (T)(threadIdx.x + c);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = x[c] * a + b;
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) s += x[c];
    if (s == (T)-1.2345) out[0] = s;   // keeps the chains alive; never true for these inputs
}

template <typename T>
static double fma_peak(int iters) {
    int dev = 0, n_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    T* out = nullptr;
    OMG_CUDA(cudaMalloc(&out, sizeof(T)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const unsigned grid = (unsigned)n_sm * 8;
    fma_peak_kernel<T><<<grid, 256>>>(iters / 10, (T)0.999, (T)0.001, out);   // warm-up
    count_launch(2);
    cudaEventRecord(e0);
    fma_peak_kernel<T><<<grid, 256>>>(iters, (T)0.999, (T)0.001, out);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    OMG_CUDA(cudaGetLastError());
    return (double)grid * 256 * 8 * iters / (ms * 1e-3);
}

}  // namespace omg

// Measurement hook (not part of the public header): FMA instructions per
// second of the FP32 (kind 0) or FP64 (kind 1) pipe of the current device.
extern "C" int omg_internal_pipe_peak(int kind, double* fma_per_s) {
    try {
        *fma_per_s = kind == 0 ? omg::fma_peak<float>(1 << 16) : omg::fma_peak<double>(1 << 12);
        return 0;
    } catch (const omg::Error& e) {
        return e.code;
    }
}

