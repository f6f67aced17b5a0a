// Gains from an explicit inverse head matrix: GainEEG and GainMEG
// (OpenMEEG/include/gain.h:60-76) as om_gain -EEG / -MEG evaluate them
// (apps/gain.cpp:65-80, 105-122): the sensor rows times the inverse first,
// then the source matrix.  The inverse comes from om_minverser
// (SymMatrix::invert, OpenMEEGMaths/include/symmatrix.h:280-300), dense or in
// SymMatrix packed-upper storage.
//
// Both products are formed transposed, Q = HMinv V^T (N x k, one column per
// sensor; HMinv is symmetric), so that every step reads whole columns:
//  - EEG: V = Head2EEGMat is sparse (3 nonzeros per electrode); column e of Q
//    is the weighted sum of the inverse's columns at the electrode's vertices,
//    gathered by one kernel (HBM-bound, 3 N reads per electrode).
//  - MEG: V = Head2MEGMat is dense; Q is an N x N x n_squids product.
// then gain = Q^T DSM (+ DS2MM).  FP64: CUDA-core FP64 GEMMs.  Mixed: the
// FP64-accurate fixed-point digit GEMM on the bf16 tensor cores (the one the
// refinement residual uses; error below 5e-13 of |Q||DSM| normwise).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "pipeline.h"

namespace omg {
template <typename T>
void gemm(int64_t M, int64_t N, int64_t K, T alpha, const T* A, int64_t lda, bool ta, const T* B, int64_t ldb, bool tb,
          T beta, T* C, int64_t ldc, cudaStream_t s, bool lower = false, int64_t row0 = 0, int64_t col0 = 0);
int64_t digits_ld(int64_t n);
void digits_columns(const double* M, int64_t n, int64_t ncol, int64_t ldm, int nd, int beta, int64_t rows_per_plane,
                    int64_t ldo, void* out, int* ex, cudaStream_t s,
                    const std::vector<std::pair<int64_t, int64_t>>* ranges = nullptr, float* lower32 = nullptr,
                    int64_t ld32 = 0);
void digit_gemm(int64_t n, int64_t k, int64_t kdim, const void* Ad, int nda, const int* rexp, const void* Xd, int ndx,
                int64_t kpad, const int* cexp, int beta, int lmax, const double* B, int64_t ldb, double sgn, double* R,
                int64_t ldr, int* err, cudaStream_t s, const char* prof_name);
void count_launch(int n);
}  // namespace omg

using namespace omg;

namespace {

inline unsigned nblk(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

void check_k(const char* what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error(OMG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    count_launch(1);
}

// Entry (i, c) of the symmetric inverse: dense column-major, or packed upper
// (i + j (j + 1) / 2 for i <= j, SymMatrix storage, symmatrix.h:55).
__device__ __forceinline__ double sym_at(const double* __restrict__ H, int64_t ld, int packed, int64_t i, int64_t c) {
    if (!packed) return H[i + c * ld];
    const int64_t a = i < c ? i : c, b = i < c ? c : i;
    return H[a + b * (b + 1) / 2];
}

// Q[:, e] = sum over the nonzeros (c, w) of row e of the sparse sensor matrix
// of w HMinv[:, c]; the nonzeros of a row are summed in their CSR order.
__global__ void gather_inverse_columns_kernel(int64_t N, const double* __restrict__ H, int64_t ld, int packed,
                                              int64_t ne, const int64_t* __restrict__ rbeg,
                                              const int64_t* __restrict__ cols, const double* __restrict__ vals,
                                              double* __restrict__ Q) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= N) return;
    for (int64_t e = blockIdx.y; e < ne; e += gridDim.y) {
        double acc = 0.0;
        for (int64_t k = rbeg[e]; k < rbeg[e + 1]; ++k) acc += vals[k] * sym_at(H, ld, packed, i, cols[k]);
        Q[i + e * N] = acc;
    }
}

// Packed upper -> dense column-major (both triangles).
__global__ void unpack_symmetric_kernel(int64_t N, const double* __restrict__ P, double* __restrict__ D) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= N) return;
    for (int64_t j = blockIdx.y; j < N; j += gridDim.y) D[i + j * N] = sym_at(P, 0, 1, i, j);
}

// B (n x m, column-major) = A^T for A m x n column-major with leading dimension lda.
__global__ void transpose_kernel(int64_t m, int64_t n, const double* __restrict__ A, int64_t lda, double* __restrict__ B) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;   // column of B = column of A^T
    if (j >= n) return;
    for (int64_t i = blockIdx.y; i < m; i += gridDim.y) B[j + i * n] = A[i + j * lda];
}

// gain (k x nd) = Q^T DSM + (init ? init : 0), Q: N x k, DSM: N x nd, both leading dimension N.
void contract(int64_t N, int64_t k, const double* Q, const double* DSM, int64_t nd, const double* init, double* gain,
              int precision, int* err, cudaStream_t s) {
    if (precision == OMG_PREC_MIXED) {
        const int ndg = 6, beta = 7, lmax = 7;
        const int64_t ld = digits_ld(N), ndpad = (nd + 127) / 128 * 128;
        DevBuf Ad((size_t)ndg * k * ld * 2, s), Xd((size_t)ndg * ndpad * ld * 2, s), ex((size_t)(k + ndpad) * 4, s);
        int* rexp = ex.as<int>();
        digits_columns(Q, N, k, N, ndg, beta, k, ld, Ad.p, rexp, s);
        digits_columns(DSM, N, nd, N, ndg, beta, ndpad, ld, Xd.p, rexp + k, s);
        if (init)
            OMG_CUDA(cudaMemcpyAsync(gain, init, (size_t)k * nd * 8, cudaMemcpyDeviceToDevice, s));
        else
            OMG_CUDA(cudaMemsetAsync(gain, 0, (size_t)k * nd * 8, s));
        digit_gemm(k, nd, N, Ad.p, ndg, rexp, Xd.p, ndg, ndpad, rexp + k, beta, lmax, gain, k, 1.0, gain, k, err, s,
                   "gain_direct_tc");
        return;
    }
    if (init) OMG_CUDA(cudaMemcpyAsync(gain, init, (size_t)k * nd * 8, cudaMemcpyDeviceToDevice, s));
    gemm<double>(k, nd, N, 1.0, Q, N, true, DSM, N, false, init ? 1.0 : 0.0, gain, k, s);
}

void check_common(omg_context ctx, int64_t N, const double* hminv, int64_t ld, int32_t packed, const double* dsm,
                  int64_t nd, int32_t precision, const double* gain) {
    OMG_REQUIRE(ctx, "null context");
    OMG_REQUIRE(N > 0, "N must be positive");
    OMG_REQUIRE(nd >= 0, "negative dipole count");
    OMG_REQUIRE(packed == 0 || packed == 1, "packed must be 0 or 1");
    OMG_REQUIRE(packed || ld >= N, "leading dimension of the inverse below N");
    OMG_REQUIRE(precision == OMG_PREC_FP64 || precision == OMG_PREC_MIXED, "unknown precision");
    OMG_REQUIRE(hminv && (nd == 0 || (dsm && gain)), "null argument");
}

}  // namespace

extern "C" int omg_gain_eeg_dev(omg_context ctx, int64_t N, const double* hminv, int64_t ld, int32_t packed,
                                const double* dsm, int64_t n_dipoles, int64_t n_electrodes, int64_t nnz,
                                const int64_t* h2em_rows, const int64_t* h2em_cols, const double* h2em_vals,
                                int32_t precision, double* gain) {
    return guarded([&] {
        check_common(ctx, N, hminv, ld, packed, dsm, n_dipoles, precision, gain);
        OMG_REQUIRE(n_electrodes >= 0 && nnz >= 0, "negative electrode or nonzero count");
        OMG_REQUIRE(nnz == 0 || (h2em_rows && h2em_cols && h2em_vals), "null sparse sensor matrix");
        set_device(ctx);
        reset_err(ctx);
        cudaStream_t s = ctx->stream;
        if (n_electrodes == 0 || n_dipoles == 0) return;
        // the sparse rows in CSR order (stable: a row's nonzeros keep their given order)
        std::vector<int64_t> r(nnz), c(nnz);
        std::vector<double> v(nnz);
        if (nnz) {
            OMG_CUDA(cudaMemcpyAsync(r.data(), h2em_rows, nnz * 8, cudaMemcpyDeviceToHost, s));
            OMG_CUDA(cudaMemcpyAsync(c.data(), h2em_cols, nnz * 8, cudaMemcpyDeviceToHost, s));
            OMG_CUDA(cudaMemcpyAsync(v.data(), h2em_vals, nnz * 8, cudaMemcpyDeviceToHost, s));
            OMG_CUDA(cudaStreamSynchronize(s));
        }
        std::vector<int64_t> beg(n_electrodes + 1, 0);
        for (int64_t k = 0; k < nnz; ++k) {
            OMG_REQUIRE(r[k] >= 0 && r[k] < n_electrodes, "sparse sensor row out of range");
            OMG_REQUIRE(c[k] >= 0 && c[k] < N, "sparse sensor column out of range");
            beg[r[k] + 1]++;
        }
        for (int64_t e = 0; e < n_electrodes; ++e) beg[e + 1] += beg[e];
        std::vector<int64_t> pos(beg.begin(), beg.end() - 1), cs(nnz);
        std::vector<double> vs(nnz);
        for (int64_t k = 0; k < nnz; ++k) {
            const int64_t p = pos[r[k]]++;
            cs[p] = c[k];
            vs[p] = v[k];
        }
        DevBuf d_beg((n_electrodes + 1) * 8, s), d_c(std::max<int64_t>(nnz, 1) * 8, s),
            d_v(std::max<int64_t>(nnz, 1) * 8, s), Q((size_t)N * n_electrodes * 8, s);
        OMG_CUDA(cudaMemcpyAsync(d_beg.p, beg.data(), (n_electrodes + 1) * 8, cudaMemcpyHostToDevice, s));
        if (nnz) {
            OMG_CUDA(cudaMemcpyAsync(d_c.p, cs.data(), nnz * 8, cudaMemcpyHostToDevice, s));
            OMG_CUDA(cudaMemcpyAsync(d_v.p, vs.data(), nnz * 8, cudaMemcpyHostToDevice, s));
        }
        {
            ProfScope prof_("gather_inverse_columns", s);
            dim3 grid(nblk(N, 256), (unsigned)std::min<int64_t>(n_electrodes, 32768));
            gather_inverse_columns_kernel<<<grid, 256, 0, s>>>(N, hminv, ld, packed, n_electrodes, d_beg.as<int64_t>(),
                                                               d_c.as<int64_t>(), d_v.as<double>(), Q.as<double>());
            check_k("gather inverse columns");
        }
        contract(N, n_electrodes, Q.as<double>(), dsm, n_dipoles, nullptr, gain, precision, ctx->d_err, s);
        check_err(ctx, "GainEEG");
    });
}

extern "C" int omg_gain_meg_dev(omg_context ctx, int64_t N, const double* hminv, int64_t ld, int32_t packed,
                                const double* dsm, int64_t n_dipoles, const double* h2mm, int64_t n_squids,
                                const double* ds2mm, int32_t precision, double* gain) {
    return guarded([&] {
        check_common(ctx, N, hminv, ld, packed, dsm, n_dipoles, precision, gain);
        OMG_REQUIRE(n_squids >= 0, "negative sensor count");
        OMG_REQUIRE(n_squids == 0 || n_dipoles == 0 || (h2mm && ds2mm), "null sensor matrices");
        set_device(ctx);
        reset_err(ctx);
        cudaStream_t s = ctx->stream;
        if (n_squids == 0 || n_dipoles == 0) return;
        const double* H = hminv;
        int64_t ldh = ld;
        DevBuf dense(packed ? (size_t)N * N * 8 : 0, s);
        if (packed) {
            ProfScope prof_("unpack_symmetric", s);
            dim3 grid(nblk(N, 256), (unsigned)std::min<int64_t>(N, 32768));
            unpack_symmetric_kernel<<<grid, 256, 0, s>>>(N, hminv, dense.as<double>());
            check_k("unpack symmetric");
            H = dense.as<double>();
            ldh = N;
        }
        DevBuf Vt((size_t)N * n_squids * 8, s), Q((size_t)N * n_squids * 8, s);
        {
            ProfScope prof_("transpose", s);
            dim3 grid(nblk(N, 256), (unsigned)std::min<int64_t>(n_squids, 32768));
            transpose_kernel<<<grid, 256, 0, s>>>(n_squids, N, h2mm, n_squids, Vt.as<double>());
            check_k("transpose");
        }
        // Q = HMinv H2MM^T (N x n_squids): HMinv is symmetric, so Q = HMinv^T Vt as well
        if (precision == OMG_PREC_MIXED) {
            const int ndg = 6, beta = 7, lmax = 7;
            const int64_t ldd = digits_ld(N), kpad = (n_squids + 127) / 128 * 128;
            DevBuf Ad((size_t)ndg * N * ldd * 2, s), Xd((size_t)ndg * kpad * ldd * 2, s), ex((size_t)(N + kpad) * 4, s);
            int* rexp = ex.as<int>();
            digits_columns(H, N, N, ldh, ndg, beta, N, ldd, Ad.p, rexp, s);
            digits_columns(Vt.as<double>(), N, n_squids, N, ndg, beta, kpad, ldd, Xd.p, rexp + N, s);
            OMG_CUDA(cudaMemsetAsync(Q.p, 0, (size_t)N * n_squids * 8, s));
            digit_gemm(N, n_squids, N, Ad.p, ndg, rexp, Xd.p, ndg, kpad, rexp + N, beta, lmax, Q.as<double>(), N, 1.0,
                       Q.as<double>(), N, ctx->d_err, s, "gain_direct_tc");
        } else {
            gemm<double>(N, n_squids, N, 1.0, H, ldh, false, Vt.as<double>(), N, false, 0.0, Q.as<double>(), N, s);
        }
        contract(N, n_squids, Q.as<double>(), dsm, n_dipoles, ds2mm, gain, precision, ctx->d_err, s);
        check_err(ctx, "GainMEG");
    });
}
