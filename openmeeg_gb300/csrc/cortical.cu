// Cortical mapping: CorticalMat and CorticalMat2 (OpenMEEG/src/assembleHeadMat.cpp:137-323).
//
// Both reference formulas are the solution of one symmetric indefinite
// (KKT) system, solved here by the FP64 LU with partial pivoting (lu.cu):
//
//   CorticalMat:  X = P pinv(P^T A P) P^T M^T, P the projector on the null
//                 space of `mat` (the head-matrix rows outside the cortex),
//                 A = M^T M + alphas RR.  With V2 an orthonormal basis of that
//                 null space, P A P = V2 (V2^T A V2) V2^T, so
//                 X = V2 (V2^T A V2)^-1 V2^T M^T, which is the X of
//                 [A mat^T; mat 0] [X; L] = [M^T; 0].
//   CorticalMat2: X = (G^-1 H^T (H G^-1 H^T)^-1) restricted to the electrode
//                 columns, H = [mat; M]: the X of [G H^T; H 0] [X; L] = [0; E]
//                 with E the last n_electrodes columns of the identity.
//
// The two agree with the reference's SVD / inverse forms whenever those are
// well posed (V2^T A V2 nonsingular, H of full row rank); the KKT form needs
// no SVD.  The gradient-norm matrix RR (Mesh::gradient_norm2, mesh.cpp:160-205)
// and M^T M are sparse and built on the host from the geometry; the dense
// system is assembled, factored and solved on the device.
#include <cmath>
#include <map>
#include <vector>

#include "pipeline.h"

namespace omg {

void lu_factor(int64_t n, double* A, int64_t lda, int* ipiv, std::vector<int64_t>& perm, int* err, cudaStream_t s);
void lu_solve(int64_t n, int64_t nrhs, const double* LU, int64_t lda, const int64_t* perm_dev, double* B, int64_t ldb,
              cudaStream_t s);
template <typename T>
void gemm(int64_t M, int64_t N, int64_t K, T alpha, const T* A, int64_t lda, bool ta, const T* B, int64_t ldb, bool tb,
          T beta, T* C, int64_t ldc, cudaStream_t s, bool lower = false, int64_t row0 = 0, int64_t col0 = 0);

namespace {

static inline void check(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error(OMG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    count_launch();
}

// K(i, j) = K(j, i) = v for the listed entries (i <= j, each once).
__global__ void scatter_sym_kernel(int64_t n, const int64_t* __restrict__ ij, const double* __restrict__ v, double* K,
                                   int64_t ld) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = ij[2 * e], j = ij[2 * e + 1];
        K[i + j * ld] = v[e];
        K[j + i * ld] = v[e];
    }
}

// Row r of `mat` into K at row r0 + r and column r0 + r (the KKT border) and,
// if rows_out, into rows_out (nl x nc, leading dimension nl).  Row r is row
// rows[r] of the symmetric S (read along its column) or, without rows, row r
// of src (nl x nc, leading dimension lds).
__global__ void place_rows_kernel(int64_t nl, int64_t nc, const int64_t* __restrict__ rows,
                                  const double* __restrict__ src, int64_t lds, double* K, int64_t ldk, int64_t r0,
                                  double* rows_out) {
    for (int64_t r = blockIdx.y; r < nl; r += gridDim.y)
        for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nc;
             c += (int64_t)gridDim.x * blockDim.x) {
            const double v = rows ? src[c + rows[r] * lds] : src[r + c * lds];
            if (K) {
                K[r0 + r + c * ldk] = v;
                K[c + (r0 + r) * ldk] = v;
            }
            if (rows_out) rows_out[r + c * nl] = v;
        }
}

// The sparse M (n_electrodes x nc, triplets) as M^T into R (rows 0..nc of
// column e, leading dimension ldr) and/or as rows r0 + e of the KKT border of K.
__global__ void place_triplets_kernel(int64_t nnz, const int64_t* __restrict__ rows, const int64_t* __restrict__ cols,
                                      const double* __restrict__ vals, double* R, int64_t ldr, double* K, int64_t ldk,
                                      int64_t r0) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = rows[e], j = cols[e];
        if (R) atomicAdd(R + j + i * ldr, vals[e]);
        if (K) {
            atomicAdd(K + r0 + i + j * ldk, vals[e]);
            atomicAdd(K + j + (r0 + i) * ldk, vals[e]);
        }
    }
}

// C += I - P (n x n; P null: C += I).
__global__ void add_complement_kernel(int64_t n, const double* __restrict__ P, double* C) {
    for (int64_t j = blockIdx.y; j < n; j += gridDim.y)
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
             i += (int64_t)gridDim.x * blockDim.x)
            C[i + j * n] += (i == j ? 1.0 : 0.0) - (P ? P[i + j * n] : 0.0);
}

// R(r0 + e, e) = 1.
__global__ void unit_columns_kernel(int64_t ne, double* R, int64_t ldr, int64_t r0) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < ne) R[r0 + e + e * ldr] = 1.0;
}

static unsigned grid_for(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 4096)); }
static dim3 grid2(int64_t ncol, int64_t nrow) {
    return dim3(grid_for(ncol), (unsigned)std::max<int64_t>(1, std::min<int64_t>(nrow, 32768)));
}

struct V3 {
    double x, y, z;
};
static V3 vat(const HostGeometry& h, int64_t v) { return {h.V[3 * v], h.V[3 * v + 1], h.V[3 * v + 2]}; }
static V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
static double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// OpenMEEG's P1gradient (mesh.h:240-242): crossprod(p1, p2) / det(p0, p1, p2).
static V3 p1grad(V3 p0, V3 p1, V3 p2) {
    const V3 c = cross(p1, p2);
    const double d = dot(p0, c);
    return {c.x / d, c.y / d, c.z / d};
}

struct Cortex {
    int mesh = -1;
    std::vector<int64_t> rows;   // reference indices of the head-matrix rows outside the cortex, in mesh order
};

static Cortex cortex_of(const HostGeometry& h, int domain) {
    OMG_REQUIRE(domain >= 0 && domain < (int)h.domains.size(), "CorticalMat: unknown domain");
    if (h.shared) throw Error(OMG_ERR_UNSUPPORTED, "CorticalMat: meshes sharing vertices are not supported");
    const Domain& d = h.domains[(size_t)domain];
    // assembleHeadMat.cpp:179-183 (om_error): one interface of one mesh around the source domain
    OMG_REQUIRE(d.ifb.size() == 1, "CorticalMat: the source domain must be bounded by a single interface");
    const auto& iface = h.ifaces[(size_t)d.ifb[0].iface];
    OMG_REQUIRE(iface.size() == 1, "CorticalMat: the cortex interface must consist of one mesh");
    for (int m = 0; m < h.nmesh; ++m)
        if (h.barrier[(size_t)m] && !h.outermost[(size_t)m])
            throw Error(OMG_ERR_UNSUPPORTED, "CorticalMat: inner current barriers are not supported");
    Cortex c;
    c.mesh = iface[0].first;
    for (int m = 0; m < h.nmesh; ++m) {   // HeadMatrix (assembleHeadMat.cpp:155-165)
        if (m == c.mesh) continue;
        for (int64_t v = h.vbeg[(size_t)m]; v < h.vbeg[(size_t)m + 1]; ++v) c.rows.push_back(h.vglob[(size_t)v]);
        if (!h.barrier[(size_t)m])
            for (int64_t t = h.tbeg[(size_t)m]; t < h.tbeg[(size_t)m + 1]; ++t) c.rows.push_back(h.tidx[(size_t)t]);
    }
    return c;
}

using Sparse = std::map<std::pair<int64_t, int64_t>, double>;   // (i <= j) -> value

// Mesh::gradient_norm2 of every mesh (mesh.cpp:160-205) in the reference's
// order of accumulation; upper entries.
static Sparse gradient_norm2(const HostGeometry& h) {
    Sparse A;
    auto at = [&](int64_t i, int64_t j) -> double& { return A[{std::min(i, j), std::max(i, j)}]; };
    static const int opp[3][2] = {{1, 2}, {2, 0}, {0, 1}};   // Triangle::edge / edges (triangle.h:86-94,154)
    std::vector<double> area((size_t)h.nt);
    std::vector<V3> nrm((size_t)h.nt), ctr((size_t)h.nt);
    for (int64_t t = 0; t < h.nt; ++t) {
        const V3 a = vat(h, h.T[3 * t]), b = vat(h, h.T[3 * t + 1]), c = vat(h, h.T[3 * t + 2]);
        const V3 n = cross(sub(b, a), sub(c, a));
        const double l = std::sqrt(dot(n, n));
        area[(size_t)t] = 0.5 * l;
        nrm[(size_t)t] = {n.x / l, n.y / l, n.z / l};
        ctr[(size_t)t] = {(a.x + b.x + c.x) / 3, (a.y + b.y + c.y) / 3, (a.z + b.z + c.z) / 3};
    }
    for (int m = 0; m < h.nmesh; ++m) {
        const int64_t t0 = h.tbeg[(size_t)m], t1 = h.tbeg[(size_t)m + 1];
        for (int64_t v = h.vbeg[(size_t)m]; v < h.vbeg[(size_t)m + 1]; ++v) {   // vertices (diagonal)
            const int64_t i = h.vglob[(size_t)v];
            for (int32_t q = h.v2t_beg[(size_t)v]; q < h.v2t_beg[(size_t)v + 1]; ++q) {
                const int64_t t = h.v2t_tri[(size_t)q];
                const int k = h.v2t_loc[(size_t)q];
                const V3 g = p1grad(vat(h, v), vat(h, h.T[3 * t + opp[k][0]]), vat(h, h.T[3 * t + opp[k][1]]));
                at(i, i) += dot(g, g) * area[(size_t)t] * area[(size_t)t];
            }
        }
        for (int64_t t = t0; t < t1; ++t) {   // edges
            const double a2 = area[(size_t)t] * area[(size_t)t];
            for (int e = 0; e < 3; ++e) {
                const int64_t v1 = h.T[3 * t + opp[e][0]], v2 = h.T[3 * t + opp[e][1]], v3 = h.T[3 * t + e];
                const int64_t i1 = h.vglob[(size_t)v1], i2 = h.vglob[(size_t)v2];
                if (i1 < i2) {
                    const V3 p1 = vat(h, v1), p2 = vat(h, v2), p3 = vat(h, v3);
                    at(i1, i2) += dot(p1grad(p1, p2, p3), p1grad(p2, p3, p1)) * a2;
                }
            }
        }
        if (!h.outermost[(size_t)m])   // P0 gradients between adjacent triangles (mesh.h:164-172, 246-248)
            for (int64_t t = t0; t < t1; ++t) {
                const int64_t it = h.tidx[(size_t)t];
                at(it, it) = 0.0;
                std::map<int64_t, int> cnt;
                std::vector<int64_t> adj;
                for (int k = 0; k < 3; ++k) {
                    const int64_t v = h.T[3 * t + k];
                    for (int32_t q = h.v2t_beg[(size_t)v]; q < h.v2t_beg[(size_t)v + 1]; ++q)
                        if (++cnt[h.v2t_tri[(size_t)q]] == 2) adj.push_back(h.v2t_tri[(size_t)q]);
                }
                for (int64_t t2 : adj) {
                    const int64_t it2 = h.tidx[(size_t)t2];
                    if (it < it2) {
                        const double nn = dot(nrm[(size_t)t], nrm[(size_t)t2]);
                        const V3 dc = sub(ctr[(size_t)t], ctr[(size_t)t2]);
                        at(it, it2) += nn * nn / dot(dc, dc) * area[(size_t)t] * area[(size_t)t2];
                    }
                }
            }
    }
    return A;
}

struct Entries {
    std::vector<int64_t> ij;
    std::vector<double> v;
    void add(int64_t i, int64_t j, double x) {
        ij.push_back(i);
        ij.push_back(j);
        v.push_back(x);
    }
};

static void scatter(const Entries& e, double* K, int64_t ld, std::vector<DevBuf>& keep, cudaStream_t s) {
    if (e.v.empty()) return;
    const int64_t* ij = upload(keep, e.ij, s);
    const double* v = upload(keep, e.v, s);
    scatter_sym_kernel<<<grid_for((int64_t)e.v.size()), 256, 0, s>>>((int64_t)e.v.size(), ij, v, K, ld);
    check("cortical scatter");
}

// The head-matrix rows outside the cortex: the head matrix assembled without
// the cortex's own block, deflated, in the reference numbering (dense N x N).
static DevBuf cortical_headmat(omg_geometry g, const omg_integrator& integ, int cortex) {
    cudaStream_t s = g->ctx->stream;
    const int64_t Ni = g->d.N, N = g->h.N;
    DevBuf tmp((size_t)Ni * Ni * 8, s);
    assemble_headmat_internal(g, integ, tmp.as<double>(), Ni, cortex);
    DevBuf hm((size_t)N * N * 8, s);
    launch_symmetrize_to_reference(g->dg, tmp.as<double>(), Ni, hm.as<double>(), N, false, s);
    return hm;
}

static void factor_solve(int64_t n, double* K, double* R, int64_t nrhs, omg_context ctx, const char* what) {
    cudaStream_t s = ctx->stream;
    DevBuf ipiv((size_t)n * sizeof(int), s);
    std::vector<int64_t> perm;
    lu_factor(n, K, n, ipiv.as<int>(), perm, ctx->d_err, s);
    int e = 0;
    OMG_CUDA(cudaMemcpyAsync(&e, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    OMG_CUDA(cudaStreamSynchronize(s));
    if (e == OMG_ERR_SINGULAR) throw Error(OMG_ERR_SINGULAR, std::string(what) + ": singular system");
    std::vector<DevBuf> keep;
    lu_solve(n, nrhs, K, n, upload(keep, perm, s), R, n, s);
    OMG_CUDA(cudaStreamSynchronize(s));
}

static void copy_triplets_host(int64_t nnz, const int64_t* r, const int64_t* c, const double* v,
                               std::vector<int64_t>& hr, std::vector<int64_t>& hc, std::vector<double>& hv,
                               cudaStream_t s) {
    hr.resize((size_t)nnz);
    hc.resize((size_t)nnz);
    hv.resize((size_t)nnz);
    if (nnz == 0) return;
    OMG_CUDA(cudaMemcpyAsync(hr.data(), r, (size_t)nnz * 8, cudaMemcpyDeviceToHost, s));
    OMG_CUDA(cudaMemcpyAsync(hc.data(), c, (size_t)nnz * 8, cudaMemcpyDeviceToHost, s));
    OMG_CUDA(cudaMemcpyAsync(hv.data(), v, (size_t)nnz * 8, cudaMemcpyDeviceToHost, s));
    OMG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

int64_t cortical_rows(omg_geometry geo, int domain) { return (int64_t)cortex_of(geo->h, domain).rows.size(); }

void corticalmat(omg_geometry geo, const omg_integrator& integ, int domain, int64_t ne, int64_t nnz,
                 const int64_t* mr, const int64_t* mc, const double* mv, double alpha, double beta,
                 const double* proj_in, double* proj_out, double* out) {
    omg_context ctx = geo->ctx;
    cudaStream_t s = ctx->stream;
    const HostGeometry& h = geo->h;
    const Cortex cx = cortex_of(h, domain);
    const int64_t Nc = h.N, Nl = (int64_t)cx.rows.size();
    std::vector<int64_t> hr, hc;
    std::vector<double> hv;
    copy_triplets_host(nnz, mr, mc, mv, hr, hc, hv, s);
    for (int64_t e = 0; e < nnz; ++e)
        OMG_REQUIRE(hr[(size_t)e] >= 0 && hr[(size_t)e] < ne && hc[(size_t)e] >= 0 && hc[(size_t)e] < Nc,
                    "CorticalMat: H2EM entry out of range");
    // M^T M (sparse: electrodes touch few unknowns)
    Sparse MM;
    {
        std::vector<std::vector<std::pair<int64_t, double>>> byrow((size_t)ne);
        for (int64_t e = 0; e < nnz; ++e) byrow[(size_t)hr[(size_t)e]].push_back({hc[(size_t)e], hv[(size_t)e]});
        for (const auto& row : byrow)
            for (const auto& a : row)
                for (const auto& b : row)
                    if (a.first <= b.first) MM[{a.first, b.first}] += a.second * b.second;
    }
    const Sparse RR = gradient_norm2(h);
    const int64_t nv = h.nvg;
    if (alpha < 0) {   // assembleHeadMat.cpp:215-223 (Frobenius norms of full symmetric matrices)
        double fm = 0.0, fr = 0.0;
        for (const auto& kv : MM) fm += (kv.first.first == kv.first.second ? 1.0 : 2.0) * kv.second * kv.second;
        for (const auto& kv : RR)
            if (kv.first.second < nv) fr += (kv.first.first == kv.first.second ? 1.0 : 2.0) * kv.second * kv.second;
        alpha = std::sqrt(fm) / (1.0e3 * std::sqrt(fr));
        beta = alpha * 50000.0;
    }
    // A = M^T M + alphas RR: alpha on the vertex rows, beta on the triangle rows (RR has no vertex-triangle entries)
    Entries A;
    {
        Sparse S = MM;
        for (const auto& kv : RR) S[kv.first] += (kv.first.first < nv ? alpha : beta) * kv.second;
        for (const auto& kv : S) A.add(kv.first.first, kv.first.second, kv.second);
    }
    std::vector<DevBuf> keep;
    const int64_t* dmr = mr;
    const int64_t* dmc = mc;
    const double* dmv = mv;
    DevBuf hm(0, s);
    if (!proj_in || proj_out) hm = cortical_headmat(geo, integ, cx.mesh);
    const int64_t* rows_dev = upload(keep, cx.rows, s);
    if (proj_out) {   // P = I - mat^T (mat mat^T)^-1 mat: the projector the reference saves
        DevBuf matb((size_t)Nl * Nc * 8, s), S((size_t)Nl * Nl * 8, s), W((size_t)Nl * Nc * 8, s);
        place_rows_kernel<<<grid2(Nc, Nl), 256, 0, s>>>(Nl, Nc, rows_dev, hm.as<double>(), Nc, nullptr, 0, 0,
                                                        matb.as<double>());
        check("cortical rows");
        gemm<double>(Nl, Nl, Nc, 1.0, matb.as<double>(), Nl, false, matb.as<double>(), Nl, true, 0.0, S.as<double>(),
                     Nl, s);
        OMG_CUDA(cudaMemcpyAsync(W.p, matb.p, (size_t)Nl * Nc * 8, cudaMemcpyDeviceToDevice, s));
        factor_solve(Nl, S.as<double>(), W.as<double>(), Nc, ctx, "CorticalMat projector");
        gemm<double>(Nc, Nc, Nl, -1.0, matb.as<double>(), Nl, true, W.as<double>(), Nl, false, 0.0, proj_out, Nc, s);
        add_complement_kernel<<<grid2(Nc, Nc), 256, 0, s>>>(Nc, nullptr, proj_out);   // + I
        check("cortical projector");
    }
    if (proj_in) {   // the cached projector: X = P (P A P + I - P)^-1 P M^T
        DevBuf Ad((size_t)Nc * Nc * 8, s), W((size_t)Nc * Nc * 8, s), C((size_t)Nc * Nc * 8, s);
        DevBuf Mt((size_t)Nc * ne * 8, s), Rb((size_t)Nc * ne * 8, s);
        OMG_CUDA(cudaMemsetAsync(Ad.p, 0, (size_t)Nc * Nc * 8, s));
        scatter(A, Ad.as<double>(), Nc, keep, s);
        gemm<double>(Nc, Nc, Nc, 1.0, Ad.as<double>(), Nc, false, proj_in, Nc, false, 0.0, W.as<double>(), Nc, s);
        gemm<double>(Nc, Nc, Nc, 1.0, proj_in, Nc, false, W.as<double>(), Nc, false, 0.0, C.as<double>(), Nc, s);
        add_complement_kernel<<<grid2(Nc, Nc), 256, 0, s>>>(Nc, proj_in, C.as<double>());
        check("cortical complement");
        OMG_CUDA(cudaMemsetAsync(Mt.p, 0, (size_t)Nc * ne * 8, s));
        if (nnz > 0) {
            place_triplets_kernel<<<grid_for(nnz), 256, 0, s>>>(nnz, dmr, dmc, dmv, Mt.as<double>(), Nc, nullptr, 0,
                                                                0);
            check("cortical M^T");
        }
        gemm<double>(Nc, ne, Nc, 1.0, proj_in, Nc, false, Mt.as<double>(), Nc, false, 0.0, Rb.as<double>(), Nc, s);
        factor_solve(Nc, C.as<double>(), Rb.as<double>(), ne, ctx, "CorticalMat");
        gemm<double>(Nc, ne, Nc, 1.0, proj_in, Nc, false, Rb.as<double>(), Nc, false, 0.0, out, Nc, s);
        return;
    }
    const int64_t nk = Nc + Nl;
    DevBuf K((size_t)nk * nk * 8, s), R((size_t)nk * ne * 8, s);
    OMG_CUDA(cudaMemsetAsync(K.p, 0, (size_t)nk * nk * 8, s));
    OMG_CUDA(cudaMemsetAsync(R.p, 0, (size_t)nk * ne * 8, s));
    scatter(A, K.as<double>(), nk, keep, s);
    if (Nl > 0) {
        place_rows_kernel<<<grid2(Nc, Nl), 256, 0, s>>>(Nl, Nc, rows_dev, hm.as<double>(), Nc, K.as<double>(), nk,
                                                        Nc, nullptr);
        check("cortical rows");
    }
    if (nnz > 0) {
        place_triplets_kernel<<<grid_for(nnz), 256, 0, s>>>(nnz, dmr, dmc, dmv, R.as<double>(), nk, nullptr, 0, 0);
        check("cortical M^T");
    }
    hm = DevBuf(0, s);
    factor_solve(nk, K.as<double>(), R.as<double>(), ne, ctx, "CorticalMat");
    OMG_CUDA(cudaMemcpy2DAsync(out, Nc * 8, R.p, nk * 8, Nc * 8, ne, cudaMemcpyDeviceToDevice, s));
}

void corticalmat2(omg_geometry geo, const omg_integrator& integ, int domain, int64_t ne, int64_t nnz,
                  const int64_t* mr, const int64_t* mc, const double* mv, double gamma, const double* rows_in,
                  double* rows_out, double* out) {
    omg_context ctx = geo->ctx;
    cudaStream_t s = ctx->stream;
    const HostGeometry& h = geo->h;
    const Cortex cx = cortex_of(h, domain);
    const int64_t Nc = h.N, Nl = (int64_t)cx.rows.size();
    std::vector<int64_t> hr, hc;
    std::vector<double> hv;
    copy_triplets_host(nnz, mr, mc, mv, hr, hc, hv, s);
    for (int64_t e = 0; e < nnz; ++e)
        OMG_REQUIRE(hr[(size_t)e] >= 0 && hr[(size_t)e] < ne && hc[(size_t)e] >= 0 && hc[(size_t)e] < Nc,
                    "CorticalMat2: H2EM entry out of range");
    // G: the gradient norms; the reference multiplies G(t1, t2) by gamma for every ordered pair of triangles of
    // a mesh that is not a current barrier (assembleHeadMat.cpp:297-303), i.e. gamma^2 off the diagonal of a
    // symmetric matrix and gamma on it
    const Sparse RR = gradient_norm2(h);
    std::vector<int> tmesh((size_t)Nc, -1);
    for (int m = 0; m < h.nmesh; ++m)
        if (!h.barrier[(size_t)m])
            for (int64_t t = h.tbeg[(size_t)m]; t < h.tbeg[(size_t)m + 1]; ++t) tmesh[(size_t)h.tidx[(size_t)t]] = m;
    Entries G;
    for (const auto& kv : RR) {
        const int64_t i = kv.first.first, j = kv.first.second;
        double v = kv.second;
        if (i >= h.nvg && j >= h.nvg && tmesh[(size_t)i] >= 0 && tmesh[(size_t)i] == tmesh[(size_t)j])
            v *= (i == j) ? gamma : gamma * gamma;
        G.add(i, j, v);
    }
    std::vector<DevBuf> keep;
    const int64_t nk = Nc + Nl + ne;
    DevBuf K((size_t)nk * nk * 8, s), R((size_t)nk * ne * 8, s);
    OMG_CUDA(cudaMemsetAsync(K.p, 0, (size_t)nk * nk * 8, s));
    OMG_CUDA(cudaMemsetAsync(R.p, 0, (size_t)nk * ne * 8, s));
    scatter(G, K.as<double>(), nk, keep, s);
    if (Nl > 0) {
        if (rows_in) {
            place_rows_kernel<<<grid2(Nc, Nl), 256, 0, s>>>(Nl, Nc, nullptr, rows_in, Nl, K.as<double>(), nk, Nc,
                                                            nullptr);
        } else {
            DevBuf hm = cortical_headmat(geo, integ, cx.mesh);
            const int64_t* rows_dev = upload(keep, cx.rows, s);
            place_rows_kernel<<<grid2(Nc, Nl), 256, 0, s>>>(Nl, Nc, rows_dev, hm.as<double>(), Nc, K.as<double>(),
                                                            nk, Nc, rows_out);
        }
        check("cortical rows");
    }
    if (nnz > 0) {
        place_triplets_kernel<<<grid_for(nnz), 256, 0, s>>>(nnz, mr, mc, mv, nullptr, 0, K.as<double>(), nk, Nc + Nl);
        check("cortical M rows");
    }
    unit_columns_kernel<<<grid_for(ne), 256, 0, s>>>(ne, R.as<double>(), nk, Nc + Nl);
    check("cortical rhs");
    factor_solve(nk, K.as<double>(), R.as<double>(), ne, ctx, "CorticalMat2");
    OMG_CUDA(cudaMemcpy2DAsync(out, Nc * 8, R.p, nk * 8, Nc * 8, ne, cudaMemcpyDeviceToDevice, s));
}

}  // namespace omg

using namespace omg;

extern "C" {

int omg_corticalmat_dev(omg_context ctx, omg_geometry geo, const omg_integrator* integ, int32_t domain,
                        int64_t n_electrodes, int64_t nnz, const int64_t* h2em_rows, const int64_t* h2em_cols,
                        const double* h2em_vals, double alpha, double beta, const double* projector_in,
                        double* projector_out, double* out) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && out, "null argument");
        OMG_REQUIRE(n_electrodes > 0 && nnz >= 0, "CorticalMat: bad sizes");
        OMG_REQUIRE(nnz == 0 || (h2em_rows && h2em_cols && h2em_vals), "null argument");
        set_device(ctx);
        reset_err(ctx);
        const omg_integrator it = integ ? *integ : default_hm_integrator();
        check_integrator(it, false);
        corticalmat(geo, it, domain, n_electrodes, nnz, h2em_rows, h2em_cols, h2em_vals, alpha, beta, projector_in,
                    projector_out, out);
        check_err(ctx, "CorticalMat");
    });
}

int omg_corticalmat2_dev(omg_context ctx, omg_geometry geo, const omg_integrator* integ, int32_t domain,
                         int64_t n_electrodes, int64_t nnz, const int64_t* h2em_rows, const int64_t* h2em_cols,
                         const double* h2em_vals, double gamma, const double* rows_in, double* rows_out,
                         double* out) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && out, "null argument");
        OMG_REQUIRE(n_electrodes > 0 && nnz >= 0, "CorticalMat2: bad sizes");
        OMG_REQUIRE(nnz == 0 || (h2em_rows && h2em_cols && h2em_vals), "null argument");
        set_device(ctx);
        reset_err(ctx);
        const omg_integrator it = integ ? *integ : default_hm_integrator();
        check_integrator(it, false);
        corticalmat2(geo, it, domain, n_electrodes, nnz, h2em_rows, h2em_cols, h2em_vals, gamma, rows_in, rows_out,
                     out);
        check_err(ctx, "CorticalMat2");
    });
}

int omg_cortical_rows(omg_geometry geo, int32_t domain, int64_t* n_rows) {
    return guarded([&] {
        OMG_REQUIRE(geo && n_rows, "null argument");
        *n_rows = cortical_rows(geo, domain);
    });
}

}  // extern "C"
