// C ABI of the GB300 forward path: contexts, geometry handles, assembly,
// the quasi-definite solver and the adjoint gain pipeline.  Host code only
// orchestrates; every numerical step runs in the kernels of bem_kernels.cu and
// dense_kernels.cu on the context's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "pipeline.h"

namespace omg {
void profile_enable(bool on);
std::vector<std::tuple<std::string, int64_t, double>> profile_collect();
// kernel launchers (bem_kernels.cu)
void launch_prepare_triangles_order(const DevGeom& g, int order, cudaStream_t s);
void launch_rows_to_reference(const DevGeom& g, int64_t ncol, const double* in, int64_t ldi, double* out, int64_t ldo,
                              cudaStream_t s);
void launch_from_reference_dense(const DevGeom& g, const double* in, int64_t ldi, double* hm, int64_t ld,
                                 cudaStream_t s);
void launch_mesh_solid_angles(const double* pts, int64_t pstride, int64_t n, int nmesh, const int64_t* tbeg_dev,
                              const double* srec, double* out, cudaStream_t s, bool screened = false);
void launch_domain_lookup(int64_t n, int nmesh, const double* sa, int ndom, int maxb, const int* dnb,
                          const int* bmesh, const int* binside, const int* borient, const int* bgrp, int forced,
                          int* dom, int* err, cudaStream_t s);
void launch_dsm(const DevGeom& g, int64_t dip0, int64_t ndc, const double* dip, const int32_t* tmesh,
                const int64_t* tidx_ref, const int* barrier, const int* orient, const int* dom, int maxb,
                const int* dnb, const int* bmesh, const int* binside, const double* dsigma, int order, int levels,
                double tol, int perm, double* out, int64_t ldo, double* p1tmp, int mixed, cudaStream_t s);
void launch_h2em(const DevGeom& g, const double* pos, int64_t ne, int nseg, const int64_t* seg, const int32_t* cand,
                 int perm, double* dense, int64_t rs, int64_t cs, int64_t col0, int64_t* scols, double* svals,
                 cudaStream_t s);
void launch_h2mm(const DevGeom& g, const double* sq, int64_t np, const int32_t* tmesh, const double* jump, int perm,
                 double* out, int64_t rs, int64_t cs, int64_t col0, double* F, cudaStream_t s,
                 double mag = kMagFactor);
void launch_ds2mm(const double* dip, int64_t nd, const double* sq, int64_t np, double* out, int64_t ldo,
                  cudaStream_t s);
void launch_fold_hm(int64_t Ng, int64_t nP, const int64_t* gbeg, const int64_t* gcopy, const double* hl, int64_t ldl,
                    double* hg, int64_t ldg, cudaStream_t s);
void launch_fold_rows(int64_t Ng, int64_t nP, const int64_t* gbeg, const int64_t* gcopy, int64_t ncol, const double* in,
                      int64_t ldi, double* out, int64_t ldo, cudaStream_t s);
void launch_fold_to_reference(int64_t Nref, int64_t nvg, int64_t nP, const int64_t* gbeg, const int64_t* gcopy,
                              int64_t ncol, const double* in, int64_t ldi, double* out, int64_t rs, int64_t cs,
                              cudaStream_t s);
void launch_partial_block(const DevGeom& g, int64_t p0, int64_t npc, const double* pts, const int* pdom,
                          const int64_t* rows, const int32_t* tmesh, const int64_t* tidx_ref, const int* barrier,
                          const int* orient, int maxb, const int* dnb, const int* bmesh, const int* binside,
                          const double* dsigma, double* p1tmp, double* out, int64_t ldo, cudaStream_t s,
                          int64_t tshift = 0);
void launch_fold_columns(int64_t nrow, int64_t Nref, int64_t nvg, int64_t nv, const int64_t* gbeg,
                         const int64_t* gcopy, const double* in, int64_t ldi, double* out, int64_t ldo,
                         cudaStream_t s);
void launch_nearest_triangle(const DevGeom& g, const double* pos, int64_t ne, int64_t ncand, const int32_t* cand,
                             int64_t* out_tri, cudaStream_t s);
void launch_eit_rows(const DevGeom& g, const int64_t* inj, int64_t nk, int64_t t2b, int64_t t2e, int64_t vb,
                     int64_t ve, bool self, bool withS, double coeffD, double coeffS, const int64_t* tidx_ref,
                     int order, double* tmp, double* R, cudaStream_t s);
void launch_eit_combine(int64_t Nref, int64_t ne, const int64_t* ebeg, const int64_t* eid, const double* ecoef,
                        int64_t k0, int64_t nk, const double* R, double* out, cudaStream_t s);
void launch_dipole_internal_pot(const double* pts, const int* pdom, const int64_t* rows, int64_t np, const double* dip,
                                const int* ddom, int64_t nd, const double* dsigma, double* out, int64_t ldo,
                                cudaStream_t s);
void launch_prepare_gg(const DevGeom& g, float* grec, cudaStream_t s);
void launch_dsm_vjp(const DevGeom& g, int64_t dip0, int64_t ndc, const double* dip, const int32_t* tmesh,
                    const int64_t* tidx_ref, const int* barrier, const int* orient, const int* dom, int maxb,
                    const int* dnb, const int* bmesh, const int* binside, const double* dsigma, int order, int levels,
                    double tol, const double* U, int64_t ldu, double* part, double* out, cudaStream_t s);
void launch_pad_identity(const DevGeom& g, double* hm, int64_t ld, cudaStream_t s);
void launch_ff_block(const DevGeom& g, const float* grec, int64_t t1b, int64_t t1e, int64_t t2b, int64_t t2e,
                     bool same, bool wantS, bool wantD12, bool wantD21, double cS, double* hm, int64_t ld,
                     double* stmp, double* d12, double* d21, int2* near, int* near_count, int near_cap, float rho,
                     int* err, cudaStream_t s);
void launch_near_pairs(const DevGeom& g, const int2* near, int count, int64_t t1b, int64_t t1e, int64_t t2b,
                       int64_t t2e, bool same, bool wantS, bool wantD12, bool wantD21, double cS, int order,
                       double* hm, int64_t ld, double* stmp, double* d12, double* d21, cudaStream_t s);
// dense_kernels.cu
template <typename T>
void gemm(int64_t M, int64_t N, int64_t K, T alpha, const T* A, int64_t lda, bool ta, const T* B, int64_t ldb, bool tb,
          T beta, T* C, int64_t ldc, cudaStream_t s, bool lower = false, int64_t row0 = 0, int64_t col0 = 0);
template <typename T>
void negate_lower(T* A, int64_t lda, int64_t n, cudaStream_t s);
template <typename T>
void negate_rows(T* B, int64_t ldb, int64_t r0, int64_t r1, int64_t n, cudaStream_t s);
template <typename Tin, typename Tout>
void copy_convert(int64_t m, int64_t n, const Tin* a, int64_t lda, Tout* b, int64_t ldb, bool lower, Tout scale,
                  cudaStream_t s);
void symmetrize(double* A, int64_t lda, int64_t n, cudaStream_t s);
void col_norms(int64_t m, int64_t n, const double* A, int64_t lda, double* out, cudaStream_t s);
void axpy_f32(int64_t m, int64_t n, const float* d, int64_t ldd, double* x, int64_t ldx, const double* colscale,
              cudaStream_t s);
void scale_to_f32(int64_t m, int64_t n, const double* r, int64_t ldr, float* b, int64_t ldb, const double* colnorm,
                  double* colscale, cudaStream_t s);
void residual_df64(int64_t M, int64_t N, int64_t K, const float* Ahi, const float* Alo, int64_t lda,
                   const float* Xhi, const float* Xlo, int64_t ldx, const double* B, int64_t ldb, double* R,
                   int64_t ldr, cudaStream_t s);
void split_f64(int64_t m, int64_t n, const double* A, int64_t lda, float* H, float* L, int64_t ldo, cudaStream_t s);
template <typename T>
void potrf(T* A, int64_t lda, int n, int* err, int64_t* err_col, int64_t col_offset, cudaStream_t s);
template <typename T>
void trsm_rows(int64_t m, int n, const T* L, int64_t ldl, T* P, int64_t ldp, cudaStream_t s);
template <typename T>
void trsm_cols(int64_t nrhs, int n, const T* L, int64_t ldl, bool trans, T* B, int64_t ldb, cudaStream_t s,
               const T* Lr = nullptr);
// tc_gemm.cu
void gemm_tf32x3(int64_t M, int64_t N, int64_t K, float alpha, const float* Ah, const float* Al, int64_t lda,
                 int64_t a_kext, int64_t a_k0, const float* Bh, const float* Bl, int64_t ldb, int64_t b_kext,
                 int64_t b_k0, float beta, float* C, int64_t ldc, bool lower, int* err, cudaStream_t s,
                 const char* prof_name = "gemm_tf32x3", int max_ctas = 0, float* Sh = nullptr, float* Sl = nullptr,
                 int64_t s_row0 = 0, int s_kpad = 0, float* Cr = nullptr, float* Xh = nullptr, float* Xl = nullptr,
                 int64_t x_row0 = 0, bool pdl = false);
void gemm_tf32x3_pair(int64_t M, int64_t N, float alpha, int64_t K1, const float* A1h, const float* A1l, int64_t lda1,
                      const float* B1h, const float* B1l, int64_t ldb1, int64_t K2, const float* A2h,
                      const float* A2l, int64_t lda2, const float* B2h, const float* B2l, int64_t ldb2, float beta,
                      float* C, int64_t ldc, bool lower, int* err, cudaStream_t s, const char* prof_name,
                      int max_ctas, float* Sh, float* Sl, int64_t s_row0, int s_kpad, bool pdl = false);
void gemm_tf32x3_grouped(const GemmOperand ops[8], const std::vector<GemmProduct>& prods, float alpha, int* err,
                         cudaStream_t s, const char* prof_name, bool pdl = false);
void split_panel_kmajor(int64_t m, int nk, int kpad, const float* P, int64_t ld, float* H, float* L,
                        cudaStream_t s);
void split_cols(int nk, int64_t ncol, int kpad, const float* X, int64_t ldx, float* H, float* L, cudaStream_t s);
void potrf_inv(float* A, int64_t lda, int n, int* err, int64_t* err_col, int64_t col_offset, float* Linv, float* Bh,
               float* Bl, cudaStream_t s, bool store_l = true, bool pdl = false);
void linv_from_split(int64_t nblocks, const float* B, float* Linv, float* LCh, float* LCl, cudaStream_t s);
void diag_update(float* A, int64_t lda, int n, const float* P0h, const float* P0l, const float* P1h, const float* P1l,
                 cudaStream_t s, bool pdl = false);
void apply_inv_blocks(int64_t nblocks, int nb, int n_last, int64_t ncol, const float* Li, bool trans, float* B,
                      int64_t ldb, cudaStream_t s);
void col_norms_f32(int64_t m, int64_t n, const float* A, int64_t lda, const double* scale, double* out,
                   cudaStream_t s);
void ratio_max(int64_t n, const double* num, const double* den, double* out, cudaStream_t s);
int64_t digits_ld(int64_t n);
void digits_columns(const double* M, int64_t n, int64_t ncol, int64_t ldm, int nd, int beta, int64_t rows_per_plane,
                    int64_t ldo, void* out, int* ex, cudaStream_t s,
                    const std::vector<std::pair<int64_t, int64_t>>* ranges = nullptr, float* lower32 = nullptr,
                    int64_t ld32 = 0);
void digit_gemm(int64_t n, int64_t k, int64_t kdim, const void* Ad, int nda, const int* rexp, const void* Xd, int ndx,
                int64_t kpad, const int* cexp, int beta, int lmax, const double* B, int64_t ldb, double sgn, double* R,
                int64_t ldr, int* err, cudaStream_t s, const char* prof_name);
// tc_solve.cu
size_t sweep_scratch_bytes(int64_t nblocks, int64_t nrhs);
void solve_sweep_tc(bool backward, int64_t N, int64_t nblocks, const float* W, int64_t w_rows, const float* A,
                    const float* Ar, int64_t ld, float* B, int64_t ldb, int64_t nrhs, void* scratch, int* err,
                    cudaStream_t s, int max_ctas = 0);
void residual_slices(int64_t n, int64_t k, const void* Ad, int nda, const int* rexp, const void* Xd, int ndx,
                     int64_t kpad, const int* cexp, int beta, int lmax, const double* B, int64_t ldb, double* R,
                     int64_t ldr, int* err, cudaStream_t s);
void launch_domain_check(int64_t n, const int* dom, uint64_t allowed, int* err, cudaStream_t s);
}  // namespace omg

using namespace omg;

static thread_local std::string g_last_error;
std::atomic<int64_t> g_dev_live{0}, g_dev_peak{0};
void set_last_error(const char* msg) { g_last_error = msg; }

void set_device(omg_context ctx) { OMG_CUDA(cudaSetDevice(ctx->device)); }

// Handles are reference counted so that destroying them in any order is safe:
// a context stays alive while a geometry or solver made from it lives, and a
// geometry while a solver built on it lives.
void release_context(omg_context ctx) {
    if (!ctx || --ctx->refs > 0) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->own);
    cudaFree(ctx->d_err);
    cudaFree(ctx->d_errcol);
    cudaFree(ctx->d_scalar);
    if (ctx->aux) cudaStreamSynchronize(ctx->aux);
    release_aux(ctx);
    if (ctx->own) cudaStreamDestroy(ctx->own);
    delete ctx;
}

static int n_sm() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// Points the context's stream at another stream for a scope (the library's calls take the context's
// stream), restoring it at scope exit.
struct StreamSwap {
    omg_context ctx;
    cudaStream_t saved;
    StreamSwap(omg_context c, cudaStream_t st) : ctx(c), saved(c->stream) { c->stream = st; }
    ~StreamSwap() { ctx->stream = saved; }
    StreamSwap(const StreamSwap&) = delete;
    StreamSwap& operator=(const StreamSwap&) = delete;
};

void ensure_aux(omg_context ctx) {
    if (!ctx->aux) OMG_CUDA(cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking));
    if (!ctx->hi) {
        int least = 0, greatest = 0;
        OMG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        OMG_CUDA(cudaStreamCreateWithPriority(&ctx->hi, cudaStreamNonBlocking, greatest));
    }
    for (cudaEvent_t* e : {&ctx->ev_a, &ctx->ev_b, &ctx->ev_c, &ctx->ev_d, &ctx->ev_e})
        if (!*e) OMG_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
}

void release_geometry(omg_geometry geo) {
    if (!geo || --geo->refs > 0) return;
    omg_context ctx = geo->ctx;
    cudaSetDevice(ctx->device);
    geo->bufs.clear();
    delete geo;
    release_context(ctx);
}

void reset_err(omg_context ctx) {
    OMG_CUDA(cudaMemsetAsync(ctx->d_err, 0, sizeof(int) * 4, ctx->stream));
    OMG_CUDA(cudaMemsetAsync(ctx->d_errcol, 0, sizeof(int64_t), ctx->stream));
}

// Synchronizes the stream and turns a device-side status into an exception.
void check_err(omg_context ctx, const char* what) {
    int h[4] = {0, 0, 0, 0};
    int64_t col = 0;
    OMG_CUDA(cudaMemcpyAsync(h, ctx->d_err, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    OMG_CUDA(cudaMemcpyAsync(&col, ctx->d_errcol, sizeof(col), cudaMemcpyDeviceToHost, ctx->stream));
    OMG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (h[0] == OMG_ERR_NOT_DEFINITE)
        throw Error(OMG_ERR_NOT_DEFINITE, std::string(what) + ": pivot of the wrong sign at internal column " +
                                              std::to_string(col) + " (head matrix not quasi-definite)");
    if (h[0] == OMG_ERR_TIMEOUT) throw Error(OMG_ERR_TIMEOUT, std::string(what) + ": a bounded device wait gave up");
    if (h[0] == OMG_ERR_INVALID)
        throw Error(OMG_ERR_INVALID, std::string(what) + ": a dipole lies in no domain of the geometry");
    if (h[0] != 0) throw Error(h[0], std::string(what) + ": device error");
}

omg_integrator default_hm_integrator() { return {3, 0, 0.005}; }      // assemble.h:32
omg_integrator default_dsm_integrator() { return {3, 10, 0.001}; }    // assembleSourceMat.h:28

void check_integrator(const omg_integrator& it, bool allow_adaptive) {
    OMG_REQUIRE(it.order >= 0 && it.order <= 3, "integrator order must be 0..3");
    OMG_REQUIRE(it.levels >= 0, "integrator levels must be >= 0");
    if (!allow_adaptive && it.levels > 0)
        throw Error(OMG_ERR_UNSUPPORTED, "adaptive integration of the head matrix is not supported");
    OMG_REQUIRE(it.levels <= 12, "adaptive integration depth is limited to 12 levels");
}

// ---------------------------------------------------------------------------
// Geometry upload
// ---------------------------------------------------------------------------

// The block of meshes (m1, m2) of the matrix (lower storage at the triangles' positions) is contiguous along
// mesh 2's index when mesh 2's triangles come after mesh 1's (a self block: along the first index).
static bool s_along_b(const HostGeometry& h, int m1, int m2) {
    return m1 != m2 && h.tidx[h.tbeg[m2]] > h.tidx[h.tbeg[m1]];
}

static void upload_geometry(omg_geometry g) {
    cudaStream_t s = g->ctx->stream;
    HostGeometry& h = g->h;
    DevGeom& d = g->d;
    d.nv = h.nv;
    d.nvg = h.nvg;
    d.nt = h.nt;
    d.nPt = h.nP;
    d.nP = (h.nP + kPad - 1) / kPad * kPad;
    d.N = d.nP + h.nv;
    d.Nref = h.N;
    d.nmesh = h.nmesh;
    d.V = upload(g->bufs, h.V, s);
    d.T = upload(g->bufs, h.T, s);
    std::vector<int32_t> tpos(h.nt, -1), tmesh(h.nt, 0);
    for (int m = 0; m < h.nmesh; ++m)
        for (int64_t t = h.tbeg[m]; t < h.tbeg[m + 1]; ++t) {
            tmesh[t] = m;
            if (!h.barrier[m]) tpos[t] = (int32_t)(h.tidx[t] - h.nvg);
        }
    d.tpos = upload(g->bufs, tpos, s);
    g->bufs.emplace_back((size_t)h.nt * SREC * 8, s, true);
    d.srec = g->bufs.back().as<double>();
    g->bufs.emplace_back((size_t)h.nt * PREC * 8, s, true);
    d.prec = g->bufs.back().as<double>();
    g->bufs.emplace_back((size_t)h.nt * QREC * 8, s, true);
    d.qrec = g->bufs.back().as<double>();
    d.v2t_beg = upload(g->bufs, h.v2t_beg, s);
    d.v2t_tri = upload(g->bufs, h.v2t_tri, s);
    d.v2t_loc = upload(g->bufs, h.v2t_loc, s);
    g->bufs.emplace_back(std::max<size_t>(1, h.v2t_tri.size()) * 3 * sizeof(double), s, true);
    d.v2t_q = g->bufs.back().as<double>();
    g->tmesh = upload(g->bufs, tmesh, s);
    g->tidx_ref = upload(g->bufs, h.tidx, s);
    g->barrier = upload(g->bufs, h.barrier, s);
    g->tbeg = upload(g->bufs, h.tbeg, s);
    if (h.shared) {   // copy -> distinct vertex, and its inverse
        d.vglob = upload(g->bufs, h.vglob, s);
        std::vector<int64_t> gb(h.nvg + 1, 0), gc(h.nv);
        for (int64_t v = 0; v < h.nv; ++v) gb[h.vglob[v] + 1]++;
        for (int64_t u = 0; u < h.nvg; ++u) gb[u + 1] += gb[u];
        std::vector<int64_t> fill(gb.begin(), gb.end() - 1);
        for (int64_t v = 0; v < h.nv; ++v) gc[fill[h.vglob[v]]++] = v;
        g->gbeg = upload(g->bufs, gb, s);
        g->gcopy = upload(g->bufs, gc, s);
    }
    g->dg = d;
    g->dg.nv = h.nvg;
    g->dg.N = d.nP + h.nvg;
    std::vector<double> jump(h.nmesh);
    for (int m = 0; m < h.nmesh; ++m) jump[m] = h.conductivity_jump(m);
    g->jump = upload(g->bufs, jump, s);
    std::vector<int32_t> cand;
    std::vector<int64_t> seg{0};   // one candidate segment per interface, in the reference's visiting order
    for (int i : h.eeg_ifaces) {
        for (const auto& om : h.ifaces[i])
            for (int64_t t = h.tbeg[om.first]; t < h.tbeg[om.first + 1]; ++t) cand.push_back((int32_t)t);
        seg.push_back((int64_t)cand.size());
    }
    g->n_eeg_seg = (int)seg.size() - 1;
    g->eeg_seg = upload(g->bufs, seg, s);
    g->n_eeg_cand = (int64_t)cand.size();
    g->eeg_cand = upload(g->bufs, cand, s);
    g->ndom = (int)h.domains.size();
    g->maxb = 1;
    for (const auto& dm : h.domains) g->maxb = std::max(g->maxb, (int)dm.bounds.size());
    std::vector<int> dnb(g->ndom), bm(g->ndom * g->maxb, -1), bi(g->ndom * g->maxb, 0), bo(g->ndom * g->maxb, 1),
        bg(g->ndom * g->maxb + 1, -1);
    std::vector<double> sig(g->ndom);
    for (int k = 0; k < g->ndom; ++k) {
        dnb[k] = (int)h.domains[k].bounds.size();
        sig[k] = h.domains[k].sigma;
        for (int j = 0; j < dnb[k]; ++j) {
            const Boundary& b = h.domains[k].bounds[j];
            bm[k * g->maxb + j] = b.mesh;
            bi[k * g->maxb + j] = b.inside ? 1 : 0;
            bo[k * g->maxb + j] = b.o;
            bg[k * g->maxb + j] = b.group;
        }
    }
    g->dnb = upload(g->bufs, dnb, s);
    g->bmesh = upload(g->bufs, bm, s);
    g->binside = upload(g->bufs, bi, s);
    g->orient = upload(g->bufs, bo, s);
    g->bgrp = upload(g->bufs, bg, s);
    g->dsigma = upload(g->bufs, sig, s);
    launch_prepare_triangles_order(d, 3, s);
    launch_prepare_vertex_curls(d, s);
    g->prepared_order = 3;
}

void ensure_order(omg_geometry g, int order) {
    if (g->prepared_order != order) {
        launch_prepare_triangles_order(g->d, order, g->ctx->stream);
        g->prepared_order = order;
    }
}

// ---------------------------------------------------------------------------
// HeadMat assembly into the internal lower triangle (assembleHeadMat.cpp:73-115)
// ---------------------------------------------------------------------------
void assemble_headmat_internal(omg_geometry g, const omg_integrator& integ, double* hm, int64_t ld,
                               int skip_self_mesh) {
    omg_context ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    const HostGeometry& h = g->h;
    const DevGeom& d = g->d;
    check_integrator(integ, false);
    ensure_order(g, integ.order);
    const int order = integ.order;
    OMG_CUDA(cudaMemsetAsync(hm, 0, sizeof(double) * (size_t)ld * (size_t)d.N, s));
    launch_pad_identity(d, hm, ld, s);
    for (const auto& p : h.pairs) {
        const int m1 = p.m1, m2 = p.m2;
        const bool same = (m1 == m2);
        if (same && m1 == skip_self_mesh) continue;
        const int64_t t1b = h.tbeg[m1], t1e = h.tbeg[m1 + 1], t2b = h.tbeg[m2], t2e = h.tbeg[m2 + 1];
        const int64_t v1b = h.vbeg[m1], v1e = h.vbeg[m1 + 1], v2b = h.vbeg[m2], v2e = h.vbeg[m2 + 1];
        double Scoeff = 0.0;
        if (same ? !h.barrier[m1] : (!h.barrier[m1] && !h.barrier[m2])) {   // set_S_block
            launch_S_block(d, t1b, t1e, t2b, t2e, same, p.cS, order, hm, ld, nullptr, ctx->d_err, s);
            Scoeff = p.cS;
        }
        if (Scoeff != 0.0) {   // set_N_block from the S already in the matrix
            launch_N_block(d, v1b, v1e, t1b, t1e, v2b, v2e, t2b, t2e, same, p.cN / Scoeff, hm, ld, nullptr, hm, s,
                           false, s_along_b(h, m1, m2));
        } else {               // ... or from a temporary unit S block (current barriers)
            DevBuf tmp((size_t)(t1e - t1b) * (t2e - t2b) * 8, s);
            launch_S_block(d, t1b, t1e, t2b, t2e, same, 1.0, order, nullptr, 0, tmp.as<double>(), ctx->d_err, s);
            launch_N_block(d, v1b, v1e, t1b, t1e, v2b, v2e, t2b, t2e, same, p.cN, nullptr, ld, tmp.as<double>(), hm, s,
                           false, true);
        }
        auto dblock = [&](int ma, int mb) {
            const int64_t tab = h.tbeg[ma], tae = h.tbeg[ma + 1], tbb = h.tbeg[mb], tbe = h.tbeg[mb + 1];
            DevBuf tmp((size_t)(tae - tab) * (tbe - tbb) * 3 * 8, s);
            launch_D_block(d, tab, tae, tbb, tbe, order, tmp.as<double>(), ctx->d_err, s);
            launch_D_gather(d, tab, tae, tbb, tbe, h.vbeg[mb], h.vbeg[mb + 1], p.cD, tmp.as<double>(), hm, ld, s);
        };
        if (!h.barrier[m1]) dblock(m1, m2);                 // set_D_block
        if (!same && !h.barrier[m2]) dblock(m2, m1);        // set_Dstar_block
    }
    // deflate (assembleHeadMat.cpp:27-60)
    for (const auto& part : h.part_outermost) {
        int64_t nb = 0, i_first = 0;
        std::vector<std::pair<int64_t, int64_t>> ranges;
        for (int m : part) {
            nb += h.vbeg[m + 1] - h.vbeg[m];
            if (i_first == 0) i_first = h.vbeg[m];
            ranges.push_back({h.vbeg[m], h.vbeg[m + 1]});
        }
        if (nb > 0) launch_deflate(d, ranges, i_first, nb, hm, ld, ctx->d_scalar, s);
    }
}


// Mixed precision: far pairs by the FP32 product rule, near pairs (centroid
// distance < kRhoFar x larger max edge) by the FP64 analytic kernels.  From
// 1.5 max edges on, the 16 x 16 rule stays within 1.1e-7 (single layer) and
// 1.5e-6 (double layer, of the sum of the absolute terms) of a twice
// subdivided rule on the config1 head (below 1.5 the double layer reaches
// 3e-3); the config1 gain error against the FP64 drop-in stays 3.0e-8 (EEG)
// and 7.1e-10 (MEG), as with a split at 2 edges.
constexpr float kRhoFar = 1.5f;

void assemble_headmat_mixed(omg_geometry g, const omg_integrator& integ, double* hm, int64_t ld, NearPlan* plan) {
    omg_context ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    const HostGeometry& h = g->h;
    const DevGeom& d = g->d;
    check_integrator(integ, false);
    OMG_REQUIRE(integ.order == 3, "mixed-precision assembly uses the 16-point rule (integrator order 3)");
    ensure_order(g, 3);
    ensure_gg_tables(g);
    OMG_CUDA(cudaMemsetAsync(hm, 0, sizeof(double) * (size_t)ld * (size_t)d.N, s));
    launch_pad_identity(d, hm, ld, s);
    const bool replay = plan && plan->recorded;
    const size_t npair = h.pairs.size();
    if (plan && !replay) {
        plan->count.assign(npair, 0);
        plan->list.clear();
        plan->counter = DevBuf(sizeof(int) * std::max<size_t>(1, npair), s, true);
    }
    DevBuf counter(replay ? 0 : sizeof(int), s);
    for (size_t pi = 0; pi < npair; ++pi) {
        const auto& p = h.pairs[pi];
        const int m1 = p.m1, m2 = p.m2;
        const bool same = (m1 == m2);
        const int64_t t1b = h.tbeg[m1], t1e = h.tbeg[m1 + 1], t2b = h.tbeg[m2], t2e = h.tbeg[m2 + 1];
        const int64_t v1b = h.vbeg[m1], v1e = h.vbeg[m1 + 1], v2b = h.vbeg[m2], v2e = h.vbeg[m2 + 1];
        const int64_t n1 = t1e - t1b, n2 = t2e - t2b;
        const bool sInHM = same ? !h.barrier[m1] : (!h.barrier[m1] && !h.barrier[m2]);
        const bool wantD12 = !h.barrier[m1];
        const bool wantD21 = !same && !h.barrier[m2];
        DevBuf stmp(sInHM ? 0 : (size_t)n1 * n2 * 8, s);
        DevBuf d12(wantD12 ? (size_t)n1 * n2 * 24 : 0, s), d21(wantD21 ? (size_t)n1 * n2 * 24 : 0, s);
        if (replay) {   // the near list of this pair is known: no read-back
            int* cnt = plan->counter.as<int>() + pi;
            const int cap = std::max(1, plan->count[pi]);
            OMG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int), s));
            launch_ff_block(d, g->grec, t1b, t1e, t2b, t2e, same, true, wantD12, wantD21, p.cS,
                            sInHM ? hm : nullptr, ld, stmp.as<double>(), d12.as<double>(), d21.as<double>(),
                            plan->list[pi].as<int2>(), cnt, cap, kRhoFar, ctx->d_err, s);
            launch_near_pairs(d, plan->list[pi].as<int2>(), plan->count[pi], t1b, t1e, t2b, t2e, same, true, wantD12,
                              wantD21, p.cS, 3, sInHM ? hm : nullptr, ld, stmp.as<double>(), d12.as<double>(),
                              d21.as<double>(), s);
        } else {
            const int64_t npairs = same ? n1 * (n1 + 1) / 2 : n1 * n2;
            int cap = (int)std::min<int64_t>(npairs, std::max<int64_t>(1 << 22, npairs / 8));
            int count = 0;
            for (int attempt = 0; attempt < 2; ++attempt) {
                DevBuf nearb((size_t)cap * sizeof(int2), s);
                OMG_CUDA(cudaMemsetAsync(counter.p, 0, sizeof(int), s));
                launch_ff_block(d, g->grec, t1b, t1e, t2b, t2e, same, true, wantD12, wantD21, p.cS,
                                sInHM ? hm : nullptr, ld, stmp.as<double>(), d12.as<double>(), d21.as<double>(),
                                nearb.as<int2>(), counter.as<int>(), cap, kRhoFar, ctx->d_err, s);
                OMG_CUDA(cudaMemcpyAsync(&count, counter.p, sizeof(int), cudaMemcpyDeviceToHost, s));
                OMG_CUDA(cudaStreamSynchronize(s));
                if (count <= cap) {
                    launch_near_pairs(d, nearb.as<int2>(), count, t1b, t1e, t2b, t2e, same, true, wantD12, wantD21,
                                      p.cS, 3, sInHM ? hm : nullptr, ld, stmp.as<double>(), d12.as<double>(),
                                      d21.as<double>(), s);
                    if (plan) {
                        plan->count[pi] = count;
                        plan->list.emplace_back(sizeof(int2) * std::max(1, count), s, true);
                        if (count > 0)
                            OMG_CUDA(cudaMemcpyAsync(plan->list.back().p, nearb.p, sizeof(int2) * count,
                                                     cudaMemcpyDeviceToDevice, s));
                    }
                    break;
                }
                cap = count;   // rerun with room for every near pair (far writes are idempotent)
            }
        }
        if (sInHM)
            launch_N_block(d, v1b, v1e, t1b, t1e, v2b, v2e, t2b, t2e, same, p.cN / p.cS, hm, ld, nullptr, hm, s,
                           false, s_along_b(h, m1, m2));
        else
            launch_N_block(d, v1b, v1e, t1b, t1e, v2b, v2e, t2b, t2e, same, p.cN, nullptr, ld, stmp.as<double>(), hm,
                           s, false, true);
        if (wantD12) launch_D_gather(d, t1b, t1e, t2b, t2e, v2b, v2e, p.cD, d12.as<double>(), hm, ld, s);
        if (wantD21) launch_D_gather(d, t2b, t2e, t1b, t1e, v1b, v1e, p.cD, d21.as<double>(), hm, ld, s);
    }
    for (const auto& part : h.part_outermost) {
        int64_t nb = 0, i_first = 0;
        std::vector<std::pair<int64_t, int64_t>> ranges;
        for (int m : part) {
            nb += h.vbeg[m + 1] - h.vbeg[m];
            if (i_first == 0) i_first = h.vbeg[m];
            ranges.push_back({h.vbeg[m], h.vbeg[m + 1]});
        }
        if (nb > 0) launch_deflate(d, ranges, i_first, nb, hm, ld, ctx->d_scalar, s);
    }
    if (plan) plan->recorded = true;
}

void ensure_gg_tables(omg_geometry g) {
    if (!g->grec) {
        g->bufs.emplace_back((size_t)g->h.nt * kFarRecFloats * sizeof(float), g->ctx->stream, true);
        g->grec = g->bufs.back().as<float>();
        launch_prepare_gg(g->d, g->grec, g->ctx->stream);
    }
}

static void assemble(omg_geometry g, const omg_integrator& integ, int precision, double* hm, int64_t ld) {
    if (precision == OMG_PREC_MIXED)
        assemble_headmat_mixed(g, integ, hm, ld);
    else
        assemble_headmat_internal(g, integ, hm, ld);
}

// The head matrix in the solver's numbering (distinct vertices, lower
// triangle, ld = dg.N): assembled on the per-mesh vertex copies and, when
// meshes share vertices, folded (P^T H P).
static DevBuf assemble_system(omg_geometry g, const omg_integrator& integ, int precision, bool persistent) {
    cudaStream_t s = g->ctx->stream;
    const int64_t Nl = g->d.N, Ng = g->dg.N;
    if (!g->h.shared) {
        DevBuf hm((size_t)Ng * Ng * 8, s, persistent);
        assemble(g, integ, precision, hm.as<double>(), Ng);
        return hm;
    }
    DevBuf hl((size_t)Nl * Nl * 8, s);
    assemble(g, integ, precision, hl.as<double>(), Nl);
    DevBuf hm((size_t)Ng * Ng * 8, s, persistent);
    launch_fold_hm(Ng, g->d.nP, g->gbeg, g->gcopy, hl.as<double>(), Nl, hm.as<double>(), Ng, s);
    return hm;
}

static void require_distinct_vertices(omg_geometry g, const char* what) {
    if (g->h.shared)
        throw Error(OMG_ERR_UNSUPPORTED, std::string(what) + " is not available for geometries whose meshes share "
                                                            "vertices");
}

// ---------------------------------------------------------------------------
// Factorization: HM = L diag(+I_P, -I_V) L^T, blocked right-looking.
// ---------------------------------------------------------------------------
template <typename T>
static void factor_ldlt(omg_solver sv, T* A, int64_t ld, int nb) {
    cudaStream_t s = sv->ctx->stream;
    const int64_t N = sv->N, nP = sv->nP;
    sv->bounds.clear();
    for (int64_t k = 0; k < N;) {
        sv->bounds.push_back(k);
        int64_t e = std::min(N, k + nb);
        if (k < nP && e > nP) e = nP;
        k = e;
    }
    sv->bounds.push_back(N);
    const size_t nblocks = sv->bounds.size() - 1;
    for (size_t b = 0; b < nblocks; ++b) {
        const int64_t k0 = sv->bounds[b], k1 = sv->bounds[b + 1], nk = k1 - k0, m = N - k1;
        if (k0 == nP) negate_lower<T>(A + k0 + k0 * ld, ld, N - k0, s);   // continue on -(vertex Schur complement)
        potrf<T>(A + k0 + k0 * ld, ld, (int)nk, sv->ctx->d_err, sv->ctx->d_errcol, k0, s);
        if (m > 0) {
            trsm_rows<T>(m, (int)nk, A + k0 + k0 * ld, ld, A + k1 + k0 * ld, ld, s);          // L21 = A21 L11^-T
            gemm<T>(m, m, nk, T(-1), A + k1 + k0 * ld, ld, false, A + k1 + k0 * ld, ld, true, T(1), A + k1 + k1 * ld,
                    ld, s, true, 0, 0);                                                          // A22 -= L21 L21^T
        }
    }
}

constexpr int NB32_TC = 128;   // tensor-core path: panel width = GEMM K = 4 x 32-element TMA chunks

// FP32 factorization with the panel solves and trailing updates on the
// tensor cores (3xTF32): each diagonal block is factored and inverted in one
// CTA, the panel is L21 = A21 L11^-T by the tcgen05 GEMM, whose epilogue
// writes L21 as TF32 heads (in A) + remainders (A32r) and its K-major split
// copy (W), and the trailing block is updated by the tcgen05 GEMM from W.  At
// the end the diagonal-block inverses are folded into the solve operators:
// W_b <- L21_b Linv_b (forward sweeps) and the block rows
// L[k0:k1, 0:k0] <- Linv_b L[k0:k1, 0:k0] in A / A32r (backward sweeps).
static void factor_ldlt_tc(omg_solver sv, float* A, int64_t ld, int nb) {
    cudaStream_t s = sv->ctx->stream;
    const int64_t N = sv->N, nP = sv->nP;
    sv->bounds.clear();
    for (int64_t k = 0; k < N;) {
        sv->bounds.push_back(k);
        int64_t e = std::min(N, k + nb);
        if (k < nP && e > nP) e = nP;
        k = e;
    }
    sv->bounds.push_back(N);
    const size_t nblocks = sv->bounds.size() - 1;
    sv->w_off.assign(nblocks + 1, 0);
    for (size_t b = 0; b < nblocks; ++b) sv->w_off[b + 1] = sv->w_off[b] + 2 * (N - sv->bounds[b + 1]) * nb;
    sv->W = DevBuf((size_t)std::max<int64_t>(1, sv->w_off[nblocks]) * sizeof(float), s, sv->persistent);
    sv->Linv32 = DevBuf((size_t)nblocks * nb * nb * sizeof(float), s, sv->persistent);
    sv->A32r = DevBuf((size_t)ld * N * sizeof(float), s, sv->persistent);
    float* Ar = sv->A32r.as<float>();
    DevBuf T((size_t)2 * std::max<int64_t>(1, N) * nb * sizeof(float), s);   // A21 split, K-major
    DevBuf Bi((size_t)2 * nblocks * nb * nb * sizeof(float), s);             // L11^-1 split, K-major, per block
    float* Th = T.as<float>();
    // Three streams.  The chain of diagonal blocks and panel solves runs on the highest-priority
    // stream (sc).  The look-ahead updates of the next panels' columns run on the main stream (s):
    // the rows below the next diagonal block, while the chain updates that block by the latest panels
    // itself (a small FP32 kernel) and factors it.  The rest of each group's trailing update
    // runs on the second stream (s2) with a few SMs left free for the other two.
    //   ev_p (sc): the first 128 rows of the latest panel solve are done (the rest follow on s)
    //   ev_q (s):  the latest panel solve is complete (all its W rows)
    //   ev_l (s):  the rows below the next diagonal block and their A21 split are ready
    //   ev_g (s):  the look-ahead update of the next group's second panel is done
    //   ev_r (s2): the rest update of the previous group is done
    ensure_aux(sv->ctx);
    cudaStream_t s2 = sv->ctx->aux, sc = sv->ctx->hi;
    cudaEvent_t ev_r = sv->ctx->ev_b, ev_p = sv->ctx->ev_c, ev_l = sv->ctx->ev_d, ev_g = sv->ctx->ev_e;
    cudaEvent_t ev_q = sv->ctx->ev_a;
    OMG_CUDA(cudaEventRecord(ev_l, s));   // the head matrix is ready
    OMG_CUDA(cudaStreamWaitEvent(sc, ev_l, 0));
    bool rest_pending = false;
    const int reserve = 24;   // SMs the rest update leaves to the chain and the look-ahead (config1 factorization:
                              // 24: 17.15-17.20 ms, 32: 17.06-17.09 (within the run-to-run spread, the trailing
                              // update on 8 fewer SMs), 40: 17.31, 16: 17.76, 48: 17.90, 12: 18.21)
    bool have_t = false;     // Th/Tl hold this panel's A21 split (written by the look-ahead update on s)
    bool wait_g = false;     // the group's second diagonal block waits for its look-ahead update (ev_g)
    bool g_recorded = false; // ev_g recorded in this call (a wait on an older record would cross a graph capture)
    const float* fp[4] = {nullptr, nullptr, nullptr, nullptr};   // panels (heads, remainders) whose update
                                                                  // of the next diagonal block is pending
    // fold of block row b for the backward solves (block row <- Linv_b x block row, heads in A, remainders in
    // A32r); run after the factorization (interleaved with the rest updates it delayed the panel chain)
    auto fold_rows = [&](size_t b, cudaStream_t st) {
        const int64_t k0 = sv->bounds[b], nk = sv->bounds[b + 1] - k0;
        const float* Rh = Bi.as<float>() + 2 * b * nb * nb;   // Linv_b split, K-major rows
        gemm_tf32x3(nk, k0, nk, 1.f, Rh, Rh + nb * nb, nb, nb, 0, A, Ar, ld, N, k0, 0.f, A + k0, ld, false,
                    sv->ctx->d_err, st, "fold_rows", 0, nullptr, nullptr, 0, 0, Ar + k0, nullptr, nullptr, 0, true);
    };
    // Panels are taken in groups of two (never across the start of the vertex part): the trailing
    // update of a group runs once with K = 256, which halves the traffic of reading and writing the
    // trailing matrix compared with one update per panel.
    std::vector<size_t> groups;
    for (size_t b = 0; b < nblocks;) {
        groups.push_back(b);
        b += (b + 1 < nblocks && sv->bounds[b + 1] != nP) ? 2 : 1;
    }
    groups.push_back(nblocks);
    auto wh = [&](size_t p) { return sv->W.as<float>() + sv->w_off[p]; };
    auto wl = [&](size_t p) { return wh(p) + (N - sv->bounds[p + 1]) * nb; };
    // C -= sum over the group's panels of W_p(rows from r0) W_p(rows from c0)^T (one or two K segments)
    auto group_update = [&](size_t gb, size_t ge, int64_t M, int64_t Nc, int64_t r0, int64_t c0, float* C, bool lower,
                            cudaStream_t st, const char* name, int max_ctas, float* Sh, float* Sl, int64_t s_row0,
                            bool pdl) {
        const int64_t o1 = sv->bounds[gb + 1], nk1 = o1 - sv->bounds[gb];
        if (ge - gb == 1) {
            gemm_tf32x3(M, Nc, nk1, -1.f, wh(gb) + (r0 - o1) * nb, wl(gb) + (r0 - o1) * nb, nb, nb, 0,
                        wh(gb) + (c0 - o1) * nb, wl(gb) + (c0 - o1) * nb, nb, nb, 0, 1.f, C, ld, lower, sv->ctx->d_err,
                        st, name, max_ctas, Sh, Sl, s_row0, nb, nullptr, nullptr, nullptr, 0, pdl);
        } else {
            const int64_t o2 = sv->bounds[gb + 2], nk2 = o2 - o1;
            gemm_tf32x3_pair(M, Nc, -1.f, nk1, wh(gb) + (r0 - o1) * nb, wl(gb) + (r0 - o1) * nb, nb,
                             wh(gb) + (c0 - o1) * nb, wl(gb) + (c0 - o1) * nb, nb, nk2, wh(gb + 1) + (r0 - o2) * nb,
                             wl(gb + 1) + (r0 - o2) * nb, nb, wh(gb + 1) + (c0 - o2) * nb, wl(gb + 1) + (c0 - o2) * nb,
                             nb, 1.f, C, ld, lower, sv->ctx->d_err, st, name, max_ctas, Sh, Sl, s_row0, nb, pdl);
        }
    };
    for (size_t g = 0; g + 1 < groups.size(); ++g) {
        const size_t gb = groups[g], ge = groups[g + 1];
        if (sv->bounds[gb] == nP) {   // continue on -(vertex Schur complement): every pending update must be in
            if (rest_pending) OMG_CUDA(cudaStreamWaitEvent(sc, ev_r, 0));
            OMG_CUDA(cudaStreamWaitEvent(sc, ev_l, 0));
            if (g_recorded) OMG_CUDA(cudaStreamWaitEvent(sc, ev_g, 0));
            negate_lower<float>(A + nP + nP * ld, ld, N - nP, sc);
            have_t = false;
            wait_g = false;
            for (auto& q : fp) q = nullptr;
        }
        for (size_t b = gb; b < ge; ++b) {
            const int64_t k0 = sv->bounds[b], k1 = sv->bounds[b + 1], nk = k1 - k0, m = N - k1;
            // L11 and L11^-1 (the inverse also serves the solves), after the pending panel updates
            if (b == gb + 1 && wait_g) OMG_CUDA(cudaStreamWaitEvent(sc, ev_g, 0));
            float* Bih = Bi.as<float>() + 2 * b * nb * nb;
            float* Bil = Bih + (size_t)nb * nb;
            // programmatic dependent launches: each starts while its predecessor on the chain drains
            if (fp[0]) diag_update(A + k0 + k0 * ld, ld, (int)nk, fp[0], fp[1], fp[2], fp[3], sc, true);
            potrf_inv(A + k0 + k0 * ld, ld, (int)nk, sv->ctx->d_err, sv->ctx->d_errcol, k0, nullptr, Bih, Bil, sc,
                      false, fp[0] != nullptr);
            for (auto& q : fp) q = nullptr;
            if (m == 0) continue;
            // L21 = A21 L11^-T on the tensor cores, written as heads (A) + remainders (A32r); its epilogue
            // also writes the K-major split of L21 (W, kept for the trailing updates and the forward solves)
            float* Tl = Th + m * nb;
            if (!have_t)
                split_panel_kmajor(m, (int)nk, nb, A + k1 + k0 * ld, ld, Th, Tl, sc);
            else
                OMG_CUDA(cudaStreamWaitEvent(sc, ev_l, 0));
            // the first 128 rows (the next diagonal block's update needs them) on the chain, the rest on s
            const int64_t mt = std::min<int64_t>(m, nb);
            gemm_tf32x3(mt, nk, nb, 1.f, Th, Tl, nb, nb, 0, Bih, Bil, nb, nb, 0, 0.f, A + k1 + k0 * ld, ld, false,
                        sv->ctx->d_err, sc, "gemm_panel", 0, wh(b), wl(b), 0, nb, Ar + k1 + k0 * ld, nullptr, nullptr,
                        0, true);
            OMG_CUDA(cudaEventRecord(ev_p, sc));
            OMG_CUDA(cudaStreamWaitEvent(s, ev_p, 0));
            if (m > mt)
                gemm_tf32x3(m - mt, nk, nb, 1.f, Th + mt * nb, Tl + mt * nb, nb, nb, 0, Bih, Bil, nb, nb, 0, 0.f,
                            A + k1 + mt + k0 * ld, ld, false, sv->ctx->d_err, s, "gemm_panel", 0, wh(b) + mt * nb,
                            wl(b) + mt * nb, 0, nb, Ar + k1 + mt + k0 * ld, nullptr, nullptr, 0, true);
            OMG_CUDA(cudaEventRecord(ev_q, s));
            have_t = false;
            if (b + 1 < ge) {   // the group's second panel: the chain updates its diagonal block by this panel,
                                // the rows below it (with their A21 split) are updated beside it on s
                const int64_t k2 = sv->bounds[b + 2], nn = k2 - k1, mr = N - k2;
                if (mr > 0) {
                    gemm_tf32x3(mr, nn, nk, -1.f, wh(b) + (k2 - k1) * nb, wl(b) + (k2 - k1) * nb, nb, nb, 0, wh(b),
                                wl(b), nb, nb, 0, 1.f, A + k2 + k1 * ld, ld, false, sv->ctx->d_err, s, "gemm_next", 0,
                                Th, Th + mr * nb, 0, nb, nullptr, nullptr, nullptr, 0, true);
                    OMG_CUDA(cudaEventRecord(ev_l, s));
                    have_t = true;
                }
                fp[0] = wh(b);
                fp[1] = wl(b);
            }
        }
        if (ge == nblocks) break;
        // look-ahead on s: the next group's columns, after the group's last panel and the rest update of
        // the previous group (whose region holds them); the chain waits for that rest update too, before
        // the next one is queued on the same event
        const size_t ng = groups[g + 2];
        OMG_CUDA(cudaStreamWaitEvent(s, ev_p, 0));
        if (rest_pending) {
            OMG_CUDA(cudaStreamWaitEvent(s, ev_r, 0));
            OMG_CUDA(cudaStreamWaitEvent(sc, ev_r, 0));
        }
        rest_pending = false;
        const bool split_diag = sv->bounds[ge] != nP;   // the vertex part is negated as a whole first
        wait_g = false;
        for (size_t p = ge; p < ng; ++p) {
            const int64_t kp0 = sv->bounds[p], kp1 = sv->bounds[p + 1], w = kp1 - kp0;
            if (p == ge && split_diag) {   // rows below the diagonal block, with their A21 split
                const int64_t Mr = N - kp1;
                if (Mr > 0)
                    group_update(gb, ge, Mr, w, kp1, kp0, A + kp1 + kp0 * ld, false, s, "gemm_next", 0, Th,
                                 Th + Mr * nb, 0, true);
                have_t = Mr > 0;
            } else {
                group_update(gb, ge, N - kp0, w, kp0, kp0, A + kp0 + kp0 * ld, false, s, "gemm_next", 0, nullptr,
                             nullptr, 0, true);
                if (p == ge) have_t = false;
            }
            OMG_CUDA(cudaEventRecord(p == ge ? ev_l : ev_g, s));
            if (p > ge) wait_g = g_recorded = true;
        }
        if (split_diag) {   // the update of the next diagonal block by this group's panels
            const int64_t kc = sv->bounds[ge];
            fp[0] = wh(gb) + (kc - sv->bounds[gb + 1]) * nb;
            fp[1] = wl(gb) + (kc - sv->bounds[gb + 1]) * nb;
            if (ge - gb == 2) {
                fp[2] = wh(gb + 1) + (kc - sv->bounds[gb + 2]) * nb;
                fp[3] = wl(gb + 1) + (kc - sv->bounds[gb + 2]) * nb;
            }
        }
        // the rest, on the second stream
        const int64_t kr = sv->bounds[ng], mr = N - kr;
        if (mr > 0) {
            OMG_CUDA(cudaStreamWaitEvent(s2, ev_q, 0));
            group_update(gb, ge, mr, mr, kr, kr, A + kr + kr * ld, true, s2, "gemm_syrk", std::max(1, n_sm() - reserve),
                         nullptr, nullptr, 0, false);
            OMG_CUDA(cudaEventRecord(ev_r, s2));
            rest_pending = true;
        }
    }
    OMG_CUDA(cudaEventRecord(ev_p, sc));
    OMG_CUDA(cudaStreamWaitEvent(s, ev_p, 0));
    if (rest_pending) OMG_CUDA(cudaStreamWaitEvent(s, ev_r, 0));
    // Fold the diagonal-block inverses into the solve operators, in place (each tile of these products
    // reads only the rows of W, or the columns of the block row, that it writes):
    //   W_b(i, c) <- sum_l L21_b(i, l) Linv_b(l, c)         as C^T = Linv_b^T W_b^T (heads in W_b, remainders
    //                                                         in its second half)
    //   A(k0 + k, m) <- sum_l Linv_b(k, l) A(k0 + l, m)      for m < k0 (heads in A, remainders in A32r)
    DevBuf LC((size_t)2 * nblocks * nb * nb * sizeof(float), s);   // Linv_b split as stored (column-major)
    float* LCh = LC.as<float>();
    float* LCl = LCh + nblocks * nb * nb;
    linv_from_split((int64_t)nblocks, Bi.as<float>(), sv->Linv32.as<float>(), LCh, LCl, s);
    if (!std::getenv("OMG_FOLD_SEPARATE")) {
        // all the folds as one grouped persistent launch (each product alone is a few latency-bound waves of
        // K = 128 tiles): the panel folds read Linv_b's split (LC) and W, the block-row folds Linv_b's K-major
        // split (Bi) and the columns of the head / remainder matrices at K offset k0
        const int64_t w_rows = sv->w_off[nblocks] / nb;
        const GemmOperand ops[8] = {{LCh, (int64_t)nblocks * nb, nb, nb},
                                    {LCl, (int64_t)nblocks * nb, nb, nb},
                                    {sv->W.as<float>(), w_rows, nb, nb},
                                    {sv->W.as<float>(), w_rows, nb, nb},
                                    {Bi.as<float>(), 2 * (int64_t)nblocks * nb, nb, nb},
                                    {Bi.as<float>(), 2 * (int64_t)nblocks * nb, nb, nb},
                                    {A, N, N, ld},
                                    {Ar, N, N, ld}};
        std::vector<GemmProduct> prods;
        prods.reserve(2 * nblocks);
        for (size_t b = 0; b < nblocks; ++b) {
            const int64_t k0 = sv->bounds[b], k1 = sv->bounds[b + 1], nk = k1 - k0, m = N - k1;
            const int64_t wr = sv->w_off[b] / nb;
            if (m > 0)   // W_b <- L21_b Linv_b
                prods.push_back(GemmProduct{wh(b), wl(b), nb, nk, m, nk, 0, (int64_t)b * nb, (int64_t)b * nb, wr,
                                            wr + m, 0, 0});
            if (k0 > 0)   // block row b <- Linv_b x block row b
                prods.push_back(GemmProduct{A + k0, Ar + k0, ld, nk, k0, nk, 1, 2 * (int64_t)b * nb,
                                            (2 * (int64_t)b + 1) * nb, 0, 0, 0, k0});
        }
        gemm_tf32x3_grouped(ops, prods, 1.f, sv->ctx->d_err, s, "fold", true);
        return;
    }
    // one launch per product (OMG_FOLD_SEPARATE=1; the grouped launch is tested against it): the panel folds
    // on the main stream, the block-row folds on the second one
    OMG_CUDA(cudaEventRecord(ev_l, s));
    OMG_CUDA(cudaStreamWaitEvent(s2, ev_l, 0));
    for (size_t b = 0; b < nblocks; ++b) {
        const int64_t k0 = sv->bounds[b], k1 = sv->bounds[b + 1], nk = k1 - k0, m = N - k1;
        if (m > 0)
            gemm_tf32x3(nk, m, nk, 1.f, LCh + b * nb * nb, LCl + b * nb * nb, nb, nb, 0, wh(b), wl(b), nb, nb, 0,
                        0.f, wh(b), nb, false, sv->ctx->d_err, s, "fold_w", 0, nullptr, nullptr, 0, 0, wl(b), nullptr,
                        nullptr, 0, true);
        if (k0 > 0) fold_rows(b, s2);
    }
    OMG_CUDA(cudaEventRecord(ev_r, s2));
    OMG_CUDA(cudaStreamWaitEvent(s, ev_r, 0));   // before the split buffers are released on the main stream
}

// FP32 solve on the tensor cores: B <- HM^-1 B (internal numbering).  With
// the diagonal-block inverses folded into W and the block rows of A, each
// sweep is a chain of tensor-core updates by the not yet inverted blocks
// (forward: b~_k = b_k - sum_{j<k} L_kj Linv_j b~_j; backward alike with
// Linv_k L_kj); the inverses are then applied to all blocks at once.  Each
// sweep runs as one persistent launch (tc_solve.cu); the fallback is one
// tensor-core update per block, each writing the K-major split of the block
// that the next update takes (band copy).  All blocks but the last have 128
// rows (the vertex part starts on a multiple of 128).
static void solve_ldlt_tc(omg_solver sv, float* B, int64_t ldb, int64_t nrhs) {
    cudaStream_t s = sv->ctx->stream;
    const int64_t N = sv->N, ld = sv->ld32;
    const float* A = sv->A32.as<float>();
    const float* Ar = sv->A32r.as<float>();
    const int nb = NB32_TC;
    const size_t nblocks = sv->bounds.size() - 1;
    for (size_t b = 0; b + 1 < nblocks; ++b)
        if (sv->bounds[b + 1] - sv->bounds[b] != nb) throw Error(OMG_ERR_UNSUPPORTED, "solver blocks not 128 wide");
    const int n_last = (int)(N - sv->bounds[nblocks - 1]);
    // W_b's heads start at K-major row 2 b N - 128 b (b + 1) (the layout the persistent sweep addresses)
    bool w_layout = true;
    for (size_t b = 0; b < nblocks; ++b)
        w_layout = w_layout && sv->w_off[b] == (2 * (int64_t)b * N - 128 * (int64_t)b * (int64_t)(b + 1)) * nb;
    if (w_layout && !std::getenv("OMG_SOLVE_CHAIN")) {
        // one persistent launch per sweep (tc_solve.cu); OMG_SOLVE_CHAIN=1 selects the chain of one
        // tensor-core update per block below (kept as the reference the sweep is tested against)
        DevBuf scratch(sweep_scratch_bytes((int64_t)nblocks, nrhs), s);
        solve_sweep_tc(false, N, (int64_t)nblocks, sv->W.as<float>(), sv->w_off[nblocks] / nb, nullptr, nullptr, 0, B,
                       ldb, nrhs, scratch.p, sv->ctx->d_err, s, sv->sweep_ctas);
        apply_inv_blocks((int64_t)nblocks, nb, n_last, nrhs, sv->Linv32.as<float>(), false, B, ldb, s);
        negate_rows<float>(B, ldb, sv->nP, N, nrhs, s);
        solve_sweep_tc(true, N, (int64_t)nblocks, nullptr, 0, A, Ar, ld, B, ldb, nrhs, scratch.p, sv->ctx->d_err, s,
                       sv->sweep_ctas);
        apply_inv_blocks((int64_t)nblocks, nb, n_last, nrhs, sv->Linv32.as<float>(), true, B, ldb, s);
        return;
    }
    const size_t xs = (size_t)nb * nrhs;
    DevBuf X(4 * xs * sizeof(float), s);
    float* xb[2] = {X.as<float>(), X.as<float>() + 2 * xs};   // heads, then remainders
    int cur = 0;
    // L y = b
    split_cols((int)std::min<int64_t>(nb, N), nrhs, nb, B, ldb, xb[0], xb[0] + xs, s);
    for (size_t b = 0; b + 1 < nblocks; ++b) {
        const int64_t k1 = sv->bounds[b + 1], nk = k1 - sv->bounds[b], m = N - k1;
        const float* Wh = sv->W.as<float>() + sv->w_off[b];
        float* xn = xb[cur ^ 1];
        gemm_tf32x3(m, nrhs, nk, -1.f, Wh, Wh + m * nb, nb, nb, 0, xb[cur], xb[cur] + xs, nb, nb, 0, 1.f, B + k1,
                    ldb, false, sv->ctx->d_err, s, "gemm_solve", 0, nullptr, nullptr, 0, 0, nullptr, xn, xn + xs, 0, true);
        cur ^= 1;
    }
    apply_inv_blocks((int64_t)nblocks, nb, n_last, nrhs, sv->Linv32.as<float>(), false, B, ldb, s);
    negate_rows<float>(B, ldb, sv->nP, N, nrhs, s);
    // L^T x = y, right-looking
    const int64_t kl = sv->bounds[nblocks - 1];
    split_cols(n_last, nrhs, nb, B + kl, ldb, xb[cur], xb[cur] + xs, s);
    for (size_t bb = nblocks - 1; bb >= 1; --bb) {
        const int64_t k0 = sv->bounds[bb], nk = sv->bounds[bb + 1] - k0;
        float* xn = xb[cur ^ 1];
        gemm_tf32x3(k0, nrhs, nk, -1.f, A, Ar, ld, N, k0, xb[cur], xb[cur] + xs, nb, nb, 0, 1.f, B, ldb, false,
                    sv->ctx->d_err, s, "gemm_solve", 0, nullptr, nullptr, 0, 0, nullptr, xn, xn + xs, k0 - nb, true);
        cur ^= 1;
    }
    apply_inv_blocks((int64_t)nblocks, nb, n_last, nrhs, sv->Linv32.as<float>(), true, B, ldb, s);
}

// In place: B <- HM^-1 B (internal numbering), HM = L diag(+I_P, -I_V) L^T.
template <typename T>
static void solve_ldlt(omg_solver sv, const T* A, int64_t ld, T* B, int64_t ldb, int64_t nrhs) {
    cudaStream_t s = sv->ctx->stream;
    const int64_t N = sv->N;
    const size_t nblocks = sv->bounds.size() - 1;
    for (size_t b = 0; b < nblocks; ++b) {   // L y = b
        const int64_t k0 = sv->bounds[b], k1 = sv->bounds[b + 1], nk = k1 - k0;
        trsm_cols<T>(nrhs, (int)nk, A + k0 + k0 * ld, ld, false, B + k0, ldb, s);
        if (k1 < N) gemm<T>(N - k1, nrhs, nk, T(-1), A + k1 + k0 * ld, ld, false, B + k0, ldb, false, T(1), B + k1, ldb, s);
    }
    negate_rows<T>(B, ldb, sv->nP, N, nrhs, s);
    // L^T x = y, right-looking: once block k is solved, remove its
    // contribution from all earlier blocks (K = block size, M = k0).
    for (size_t bb = nblocks; bb-- > 0;) {
        const int64_t k0 = sv->bounds[bb], k1 = sv->bounds[bb + 1], nk = k1 - k0;
        trsm_cols<T>(nrhs, (int)nk, A + k0 + k0 * ld, ld, true, B + k0, ldb, s);
        if (k0 > 0) gemm<T>(k0, nrhs, nk, T(-1), A + k0, ld, true, B + k0, ldb, false, T(1), B, ldb, s);
    }
}

constexpr int NB64 = 128;   // FP64 diagonal block (128 x 129 x 8 B of shared memory)
constexpr int NB32 = 128;   // FP32 diagonal block

// A current barrier that encloses a non-conductive hole (a barrier mesh that is
// not outermost, geometry.cpp:424-461) leaves the constant potential on its
// vertices in the head matrix's null space: the N block of a closed mesh and
// the solid angles the D blocks sum to both vanish on it, and the reference
// deflates only the outermost meshes (assembleHeadMat.cpp:27-60), so its head
// matrix is singular there.  The solver deflates each such mesh as the
// reference deflates an outermost one (M(v1, v2) += M(i0, i0) / n over the
// mesh's vertex block), which selects the solution orthogonal to that
// constant and changes nothing else; sensor rows and the gains do not see the
// direction.  The HeadMat returned to callers is left as the reference's.
static void deflate_enclosed_barriers(omg_solver sv, double* hm, int64_t ld) {
    const HostGeometry& h = sv->geo->h;
    if (h.shared) return;   // vertex blocks of meshes are contiguous only without shared vertices
    for (int m = 0; m < h.nmesh; ++m) {
        if (!h.barrier[m] || h.outermost[m]) continue;
        const int64_t nb = h.vbeg[m + 1] - h.vbeg[m];
        if (nb > 0)
            launch_deflate(sv->geo->d, {{h.vbeg[m], h.vbeg[m + 1]}}, h.vbeg[m], nb, hm, ld, sv->ctx->d_scalar,
                           sv->ctx->stream);
    }
}

// Factor the internal-order HeadMat held in `hm` (FP64, lower), taking ownership.
void solver_factor(omg_solver sv, DevBuf&& hm, bool check) {
    cudaStream_t s = sv->ctx->stream;
    const int64_t N = sv->N;
    if (check) reset_err(sv->ctx);   // unchecked (captured) factorizations keep earlier flags
    deflate_enclosed_barriers(sv, hm.as<double>(), N);
    if (sv->precision == OMG_PREC_FP64) {
        sv->A64 = std::move(hm);
        factor_ldlt<double>(sv, sv->A64.as<double>(), N, NB64);
    } else {
        sv->ld32 = (N + 31) / 32 * 32;
        sv->A32 = DevBuf((size_t)sv->ld32 * N * sizeof(float), s, sv->persistent);
        symmetrize(hm.as<double>(), N, N, s);
        const char* mode = std::getenv("OMG_RESIDUAL");
        sv->tc_residual = sv->residual_choice >= 0 ? sv->residual_choice == 1
                                                   : !(mode && std::string(mode) == "df64");
        if (sv->tc_residual && sv->residual_choice < 0) {
            // the digits (nda planes of N x ld bf16) must fit beside the FP32 factor's panel copies and
            // remainders (2 x 4 N^2 bytes, allocated once the FP64 matrix is gone); else the double-float
            // residual from a float pair (8 N^2 bytes) is used
            size_t free_b = 0, total_b = 0;
            OMG_CUDA(cudaMemGetInfo(&free_b, &total_b));
            const double dig = (double)sv->nda * N * digits_ld(N) * 2, later = 8.0 * N * N, margin = 4e9;
            const double after_release = (double)free_b - dig + 8.0 * N * N;
            if ((double)free_b < dig + margin || after_release < later + margin) sv->tc_residual = false;
        }
        if (sv->tc_residual) {
            // the FP64 matrix is kept only as fixed-point digits for the tensor-core residual
            const int64_t ldd = digits_ld(N);
            sv->Adig = DevBuf((size_t)sv->nda * N * ldd * 2, s, sv->persistent);
            sv->rexp = DevBuf((size_t)N * sizeof(int), s, sv->persistent);
            // (the same pass over the columns writes the FP32 lower triangle to be factored)
            digits_columns(hm.as<double>(), N, N, N, sv->nda, sv->beta, N, ldd, sv->Adig.p, sv->rexp.as<int>(), s,
                           nullptr, sv->A32.as<float>(), sv->ld32);
        } else {
            // ... or as an exact float pair (hi + lo) for the double-float residual
            copy_convert<double, float>(N, N, hm.as<double>(), N, sv->A32.as<float>(), sv->ld32, true, 1.0f, s);
            sv->A64 = DevBuf((size_t)2 * N * N * sizeof(float), s, sv->persistent);
            split_f64(N, N, hm.as<double>(), N, sv->A64.as<float>(), sv->A64.as<float>() + (size_t)N * N, N, s);
        }
        hm.release();
        factor_ldlt_tc(sv, sv->A32.as<float>(), sv->ld32, NB32_TC);
    }
    if (check) check_err(sv->ctx, "factorization");
}

namespace omg {
void lu_factor(int64_t n, double* A, int64_t lda, int* ipiv, std::vector<int64_t>& perm, int* err, cudaStream_t s);
void lu_solve(int64_t n, int64_t nrhs, const double* LU, int64_t lda, const int64_t* perm_dev, double* B, int64_t ldb,
              cudaStream_t s);
}  // namespace omg

void solver_factor_or_pivot(omg_solver sv, DevBuf&& hm, const std::function<DevBuf()>& again) {
    try {
        solver_factor(sv, std::move(hm));
        return;
    } catch (const Error& e) {
        if (e.code != OMG_ERR_NOT_DEFINITE) throw;
    }
    // a pivot of the wrong sign: the whole matrix, rebuilt, by LU with partial pivoting in FP64
    cudaStream_t s = sv->ctx->stream;
    sv->A64.release();
    sv->A32.release();
    sv->A32r.release();
    sv->W.release();
    sv->Linv32.release();
    sv->Adig.release();
    sv->rexp.release();
    sv->w_off.clear();
    reset_err(sv->ctx);
    DevBuf A = again();
    const int64_t N = sv->N;
    deflate_enclosed_barriers(sv, A.as<double>(), N);
    symmetrize(A.as<double>(), N, N, s);
    DevBuf ipiv((size_t)N * sizeof(int), s);
    std::vector<int64_t> perm;
    lu_factor(N, A.as<double>(), N, ipiv.as<int>(), perm, sv->ctx->d_err, s);
    sv->perm = DevBuf((size_t)N * sizeof(int64_t), s, sv->persistent);
    OMG_CUDA(cudaMemcpyAsync(sv->perm.p, perm.data(), (size_t)N * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    sv->A64 = std::move(A);
    sv->lu = true;
    int e = 0;
    OMG_CUDA(cudaMemcpyAsync(&e, sv->ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    OMG_CUDA(cudaStreamSynchronize(s));
    if (e == OMG_ERR_SINGULAR) throw Error(OMG_ERR_SINGULAR, "factorization: the head matrix is singular");
    check_err(sv->ctx, "pivoted factorization");
}

// Scratch of one refinement residual: X digits + column exponents, or X as a float pair.
static size_t mixed_residual_scratch(omg_solver sv, int64_t nrhs) {
    const int64_t N = sv->N;
    if (!sv->tc_residual) return (size_t)2 * N * nrhs * 4;
    const int64_t kpad = (nrhs + 127) / 128 * 128;
    return (size_t)sv->ndx * kpad * digits_ld(N) * 2 + (size_t)kpad * sizeof(int);
}

// r = B - HM x with FP64-level accuracy (x: N x nrhs, column-major).
static void mixed_residual(omg_solver sv, const double* x, int64_t nrhs, const double* B, int64_t ldb, double* r,
                           DevBuf& XS) {
    cudaStream_t s = sv->ctx->stream;
    const int64_t N = sv->N;
    if (sv->tc_residual) {
        const int64_t kpad = (nrhs + 127) / 128 * 128, ldd = digits_ld(N);
        uint8_t* xd = XS.as<uint8_t>();
        int* cexp = reinterpret_cast<int*>(xd + (size_t)sv->ndx * kpad * ldd * 2);
        digits_columns(x, N, nrhs, N, sv->ndx, sv->beta, kpad, ldd, xd, cexp, s);
        residual_slices(N, nrhs, sv->Adig.p, sv->nda, sv->rexp.as<int>(), xd, sv->ndx, kpad, cexp, sv->beta,
                        sv->lmax, B, ldb, r, N, sv->ctx->d_err, s);
    } else {
        float* xh = XS.as<float>();
        split_f64(N, nrhs, x, N, xh, xh + (size_t)N * nrhs, N, s);
        const float* ah = sv->A64.as<float>();
        residual_df64(N, nrhs, N, ah, ah + (size_t)N * N, N, xh, xh + (size_t)N * nrhs, N, B, ldb, r, N, s);
    }
}

// Mixed precision: x = HM^-1 b by FP32 solves refined against the FP64 HM.
// x0 = A32^-1 b; then r = b - A x (FP64-accurate residual), d = A32^-1 r,
// x += d, until the predicted error of x (the largest relative column
// correction times the contraction factor of the iteration) is below
// refine_tol.
static void solve_mixed(omg_solver sv, double* B, int64_t ldb, int64_t nrhs) {
    cudaStream_t s = sv->ctx->stream;
    const int64_t N = sv->N;
    DevBuf X((size_t)N * nrhs * 8, s), R((size_t)N * nrhs * 8, s), B32((size_t)N * nrhs * 4, s),
        XS(mixed_residual_scratch(sv, nrhs), s);
    DevBuf rn((size_t)nrhs * 8, s), sc((size_t)nrhs * 8, s), dn((size_t)nrhs * 8, s), xn((size_t)nrhs * 8, s),
        bn((size_t)nrhs * 8, s);
    double* x = X.as<double>();
    double* r = R.as<double>();
    OMG_CUDA(cudaMemsetAsync(x, 0, (size_t)N * nrhs * 8, s));
    copy_convert<double, double>(N, nrhs, B, ldb, r, N, false, 1.0, s);
    col_norms(N, nrhs, r, N, bn.as<double>(), s);
    std::vector<double> hb(nrhs), hr(nrhs, 0.0), hd(nrhs), hx(nrhs);
    OMG_CUDA(cudaMemcpyAsync(hb.data(), bn.p, nrhs * 8, cudaMemcpyDeviceToHost, s));
    const double* cn = bn.as<double>();
    int steps = 0;
    double last_res = 1.0, est = 1.0, prev_est = 1e300;
    for (int it = 0; it <= sv->max_refine; ++it) {
        if (it > 0) {   // r = b - HM x
            mixed_residual(sv, x, nrhs, B, ldb, r, XS);
            col_norms(N, nrhs, r, N, rn.as<double>(), s);
            cn = rn.as<double>();
            ++steps;
        }
        scale_to_f32(N, nrhs, r, N, B32.as<float>(), N, cn, sc.as<double>(), s);
        solve_ldlt_tc(sv, B32.as<float>(), N, nrhs);
        axpy_f32(N, nrhs, B32.as<float>(), N, x, N, sc.as<double>(), s);
        col_norms_f32(N, nrhs, B32.as<float>(), N, sc.as<double>(), dn.as<double>(), s);
        col_norms(N, nrhs, x, N, xn.as<double>(), s);
        OMG_CUDA(cudaMemcpyAsync(hd.data(), dn.p, nrhs * 8, cudaMemcpyDeviceToHost, s));
        OMG_CUDA(cudaMemcpyAsync(hx.data(), xn.p, nrhs * 8, cudaMemcpyDeviceToHost, s));
        if (it > 0) OMG_CUDA(cudaMemcpyAsync(hr.data(), rn.p, nrhs * 8, cudaMemcpyDeviceToHost, s));
        OMG_CUDA(cudaStreamSynchronize(s));
        est = 0.0;
        last_res = 0.0;
        for (int64_t j = 0; j < nrhs; ++j) {
            if (hx[j] > 0) est = std::max(est, hd[j] / hx[j]);
            if (it > 0 && hb[j] > 0) last_res = std::max(last_res, hr[j] / hb[j]);
        }
        // The error left in x after this correction is about est times the contraction factor of the
        // refinement, estimated as est / (the previous correction) (est_0 = 1: the first solve starts from 0).
        if (it > 0) {
            const double rho = std::min(1.0, est / (it == 1 ? 1.0 : prev_est));
            if (!(est * rho > sv->refine_tol)) {
                est *= rho;   // reported: the predicted relative error of x
                break;
            }
        }
        if (it > 1 && !(est < prev_est)) break;   // stagnation: report below
        prev_est = est;
    }
    sv->last_steps = steps;
    sv->last_residual = last_res;
    sv->last_correction = est;
    copy_convert<double, double>(N, nrhs, x, N, B, ldb, false, 1.0, s);
    if (est > sv->refine_tol)
        throw Error(OMG_ERR_NOT_CONVERGED, "iterative refinement stalled at relative correction " + std::to_string(est));
}

// Mixed solve with a fixed number of residual steps and no host read-back
// (stream-capture safe): the max relative column size of the last correction
// and of the one before it are left in d_est[0] and d_est[1] for the caller to
// test after the stream completes (predicted error d_est[0] * d_est[0] / d_est[1]).
void solve_mixed_fixed(omg_solver sv, double* B, int64_t ldb, int64_t nrhs, int residual_steps, double* d_est) {
    cudaStream_t s = sv->ctx->stream;
    const int64_t N = sv->N;
    DevBuf X((size_t)N * nrhs * 8, s), R((size_t)N * nrhs * 8, s), B32((size_t)N * nrhs * 4, s),
        XS(mixed_residual_scratch(sv, nrhs), s);
    DevBuf rn((size_t)nrhs * 8, s), sc((size_t)nrhs * 8, s), dn((size_t)nrhs * 8, s), xn((size_t)nrhs * 8, s);
    double* x = X.as<double>();
    double* r = R.as<double>();
    OMG_CUDA(cudaMemsetAsync(x, 0, (size_t)N * nrhs * 8, s));
    copy_convert<double, double>(N, nrhs, B, ldb, r, N, false, 1.0, s);
    col_norms(N, nrhs, r, N, rn.as<double>(), s);
    for (int it = 0; it <= residual_steps; ++it) {
        if (it > 0) {
            mixed_residual(sv, x, nrhs, B, ldb, r, XS);
            col_norms(N, nrhs, r, N, rn.as<double>(), s);
        }
        scale_to_f32(N, nrhs, r, N, B32.as<float>(), N, rn.as<double>(), sc.as<double>(), s);
        solve_ldlt_tc(sv, B32.as<float>(), N, nrhs);
        axpy_f32(N, nrhs, B32.as<float>(), N, x, N, sc.as<double>(), s);
        if (it + 1 >= residual_steps) {   // the last two corrections (the first, from x = 0, has size 1)
            col_norms_f32(N, nrhs, B32.as<float>(), N, sc.as<double>(), dn.as<double>(), s);
            col_norms(N, nrhs, x, N, xn.as<double>(), s);
            ratio_max(nrhs, dn.as<double>(), xn.as<double>(), d_est + (it == residual_steps ? 0 : 1), s);
        }
    }
    if (residual_steps == 0) OMG_CUDA(cudaMemcpyAsync(d_est + 1, d_est, sizeof(double), cudaMemcpyDeviceToDevice, s));
    copy_convert<double, double>(N, nrhs, x, N, B, ldb, false, 1.0, s);
}

// A stalled mixed refinement: the head matrix rebuilt and factored in FP64 (LDL^T, or the pivoted LU), the
// right-hand sides solved again from their saved copy.
static void solve_mixed_or_fp64(omg_solver sv, double* B, int64_t ldb, int64_t nrhs) {
    cudaStream_t s = sv->ctx->stream;
    const int64_t N = sv->N;
    DevBuf B0(sv->rebuild ? (size_t)N * nrhs * 8 : 0, s);
    if (sv->rebuild) OMG_CUDA(cudaMemcpy2DAsync(B0.p, N * 8, B, ldb * 8, N * 8, nrhs, cudaMemcpyDeviceToDevice, s));
    try {
        solve_mixed(sv, B, ldb, nrhs);
        return;
    } catch (const Error& e) {
        if (e.code != OMG_ERR_NOT_CONVERGED || !sv->rebuild) throw;
    }
    sv->A32.release();
    sv->A32r.release();
    sv->W.release();
    sv->Linv32.release();
    sv->Adig.release();
    sv->rexp.release();
    sv->A64.release();
    sv->w_off.clear();
    sv->precision = OMG_PREC_FP64;
    solver_factor_or_pivot(sv, sv->rebuild(), sv->rebuild);
    OMG_CUDA(cudaMemcpy2DAsync(B, ldb * 8, B0.p, N * 8, N * 8, nrhs, cudaMemcpyDeviceToDevice, s));
    solver_solve_internal(sv, B, ldb, nrhs);
}

void solver_solve_internal(omg_solver sv, double* B, int64_t ldb, int64_t nrhs) {
    if (nrhs <= 0) return;
    if (sv->lu) {
        lu_solve(sv->N, nrhs, sv->A64.as<double>(), sv->N, sv->perm.as<int64_t>(), B, ldb, sv->ctx->stream);
        sv->last_steps = 0;
        sv->last_residual = 0.0;
        sv->last_correction = 0.0;
    } else if (sv->precision == OMG_PREC_FP64)
        solve_ldlt<double>(sv, sv->A64.as<double>(), sv->N, B, ldb, nrhs);
    else
        solve_mixed_or_fp64(sv, B, ldb, nrhs);
}

// ---------------------------------------------------------------------------
// Sources / sensors
// ---------------------------------------------------------------------------
// Meshes whose rows of the DipSourceMat can be nonzero: the boundaries of the dipoles' domains (host copy of the
// per-dipole domain indices).
static std::vector<int> meshes_of_domains(omg_geometry g, const std::vector<int>& hdom) {
    std::vector<char> used(g->h.nmesh, 0);
    for (int d : hdom)
        if (d >= 0 && g->h.domains[d].sigma != 0.0)
            for (const auto& b : g->h.domains[d].bounds) used[b.mesh] = 1;
    std::vector<int> out;
    for (int m = 0; m < g->h.nmesh; ++m)
        if (used[m]) out.push_back(m);
    return out;
}

void dsm_internal(omg_geometry g, const double* dip, int64_t nd, const omg_integrator& integ, int domain, int perm,
                  double* out, int64_t ldo, int precision, std::vector<int>* meshes_used, uint64_t allowed_domains,
                  DevBuf* dom_out) {
    omg_context ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    check_integrator(integ, true);
    OMG_REQUIRE(domain >= -1 && domain < g->ndom, "domain index out of range");
    const int64_t rows = perm ? g->dg.N : g->h.N;
    if (ldo == rows)
        OMG_CUDA(cudaMemsetAsync(out, 0, (size_t)rows * nd * 8, s));
    else
        for (int64_t j = 0; j < nd; ++j) OMG_CUDA(cudaMemsetAsync(out + j * ldo, 0, (size_t)rows * 8, s));
    if (nd == 0) return;
    // meshes sharing vertices: rows on the vertex copies (internal numbering), summed per distinct vertex below
    DevBuf loc;
    double* dst = out;
    int64_t ldd = ldo;
    int dperm = perm;
    if (g->h.shared) {
        loc = DevBuf((size_t)g->d.N * nd * 8, s);
        OMG_CUDA(cudaMemsetAsync(loc.p, 0, (size_t)g->d.N * nd * 8, s));
        dst = loc.as<double>();
        ldd = g->d.N;
        dperm = 1;
    }
    DevBuf sa((size_t)nd * g->h.nmesh * 8, s), dom((size_t)nd * sizeof(int), s);
    launch_mesh_solid_angles(dip, 6, nd, g->h.nmesh, g->tbeg, g->d.srec, sa.as<double>(), s,
                             precision == OMG_PREC_MIXED);
    launch_domain_lookup(nd, g->h.nmesh, sa.as<double>(), g->ndom, g->maxb, g->dnb, g->bmesh, g->binside, g->orient,
                         g->bgrp, domain, dom.as<int>(), ctx->d_err, s);
    if (allowed_domains) launch_domain_check(nd, dom.as<int>(), allowed_domains, ctx->d_err, s);
    if (meshes_used) {   // which meshes carry nonzero DSM rows: boundaries of the dipoles' domains
        std::vector<int> hdom(nd);
        OMG_CUDA(cudaMemcpyAsync(hdom.data(), dom.p, nd * sizeof(int), cudaMemcpyDeviceToHost, s));
        OMG_CUDA(cudaStreamSynchronize(s));
        *meshes_used = meshes_of_domains(g, hdom);
    }
    // chunk the dipoles so the P1 scratch stays near 512 MB
    const int64_t per = std::max<int64_t>(1, std::min<int64_t>(4096, (512ll << 20) / (g->h.nt * 24)));
    DevBuf p1((size_t)std::min(per, nd) * g->h.nt * 24, s);
    for (int64_t d0 = 0; d0 < nd; d0 += per) {
        const int64_t n = std::min(per, nd - d0);
        launch_dsm(g->d, d0, n, dip, g->tmesh, g->tidx_ref, g->barrier, g->orient, dom.as<int>(), g->maxb, g->dnb,
                   g->bmesh, g->binside, g->dsigma, integ.order, integ.levels, integ.tol, dperm, dst, ldd,
                   p1.as<double>(), precision == OMG_PREC_MIXED ? 1 : 0, s);
    }
    if (g->h.shared) {
        if (perm)
            launch_fold_rows(g->dg.N, g->d.nP, g->gbeg, g->gcopy, nd, loc.as<double>(), g->d.N, out, ldo, s);
        else
            launch_fold_to_reference(g->h.N, g->h.nvg, g->d.nP, g->gbeg, g->gcopy, nd, loc.as<double>(), g->d.N, out,
                                     1, ldo, s);
    }
    if (dom_out) *dom_out = std::move(dom);   // the per-dipole domains, for a read-back by the caller
}

std::vector<std::pair<int64_t, int64_t>> gain_row_ranges(omg_geometry geo, const std::vector<int>& src_meshes) {
    if (geo->h.shared) return {{0, geo->dg.N}};   // vertex rows of a mesh are not contiguous
    std::vector<std::pair<int64_t, int64_t>> kr;
    for (int m : src_meshes) {
        if (!geo->h.barrier[m])
            kr.push_back({geo->h.tidx[geo->h.tbeg[m]] - geo->h.nvg, geo->h.tidx[geo->h.tbeg[m]] - geo->h.nvg +
                                                                       (geo->h.tbeg[m + 1] - geo->h.tbeg[m])});
        kr.push_back({geo->d.nP + geo->h.vbeg[m], geo->d.nP + geo->h.vbeg[m + 1]});
    }
    std::sort(kr.begin(), kr.end());
    std::vector<std::pair<int64_t, int64_t>> merged;
    for (const auto& r : kr) {
        if (!merged.empty() && r.first <= merged.back().second)
            merged.back().second = std::max(merged.back().second, r.second);
        else
            merged.push_back(r);
    }
    return merged;
}

void gain_contract(const std::vector<std::pair<int64_t, int64_t>>& merged, const double* Y, int64_t N, int64_t ne,
                   int64_t nm, const double* DSM, int64_t nd, double* geeg, double* gmeg, cudaStream_t s,
                   int precision, int* err) {
    int64_t kdim = 0;
    for (const auto& r : merged) kdim += r.second - r.first;
    const int64_t k = ne + nm;
    if (precision == OMG_PREC_MIXED && nd > 0 && k > 0 && kdim > 0 && merged.size() <= 8) {
        // FP64-level contraction on the tensor cores from fixed-point digits of Y^T and DSM (the solver's
        // digits: 6 of 7 bits each, pairs up to level 7), over the source rows only
        const int ndg = 6, beta = 7, lmax = 7;
        const int64_t ld = digits_ld(kdim), ndpad = (nd + 127) / 128 * 128;
        DevBuf Ad((size_t)ndg * k * ld * 2, s), Xd((size_t)ndg * ndpad * ld * 2, s);
        DevBuf ex((size_t)(k + ndpad) * sizeof(int), s), G((size_t)k * nd * 8, s);
        int* rexp = ex.as<int>();
        int* cexp = rexp + k;
        double* g = G.as<double>();
        digits_columns(Y, kdim, k, N, ndg, beta, k, ld, Ad.p, rexp, s, &merged);
        digits_columns(DSM, kdim, nd, N, ndg, beta, ndpad, ld, Xd.p, cexp, s, &merged);
        OMG_CUDA(cudaMemsetAsync(g, 0, (size_t)k * nd * 8, s));
        if (nm > 0)   // MEG rows start from DipSource2MEGMat
            OMG_CUDA(cudaMemcpy2DAsync(g + ne, k * 8, gmeg, nm * 8, nm * 8, nd, cudaMemcpyDeviceToDevice, s));
        digit_gemm(k, nd, kdim, Ad.p, ndg, rexp, Xd.p, ndg, ndpad, cexp, beta, lmax, g, k, 1.0, g, k, err, s,
                   "gain_tc");
        if (ne > 0) OMG_CUDA(cudaMemcpy2DAsync(geeg, ne * 8, g, k * 8, ne * 8, nd, cudaMemcpyDeviceToDevice, s));
        if (nm > 0) OMG_CUDA(cudaMemcpy2DAsync(gmeg, nm * 8, g + ne, k * 8, nm * 8, nd, cudaMemcpyDeviceToDevice, s));
        return;
    }
    if (ne > 0 && nd > 0) {
        if (merged.empty()) OMG_CUDA(cudaMemsetAsync(geeg, 0, (size_t)ne * nd * 8, s));
        for (size_t q = 0; q < merged.size(); ++q) {
            const int64_t r0 = merged[q].first, kk = merged[q].second - merged[q].first;
            gemm<double>(ne, nd, kk, 1.0, Y + r0, N, true, DSM + r0, N, false, q == 0 ? 0.0 : 1.0, geeg, ne, s);
        }
    }
    if (nm > 0 && nd > 0)
        for (const auto& r : merged)
            gemm<double>(nm, nd, r.second - r.first, 1.0, Y + ne * N + r.first, N, true, DSM + r.first, N, false, 1.0,
                         gmeg, nm, s);
}

// A geometry's meshes plus one source surface (SurfSourceMat, SurfSource2MEGMat) as
// one device geometry: the source's vertices and triangles follow the head's,
// its triangles carry no unknown, so the block kernels of the head matrix run
// between a head mesh and the source unchanged.  geo == nullptr: the source alone.
struct SourceSurface {
    DevGeom d;
    std::vector<DevBuf> bufs;
    int64_t nv0 = 0, nt0 = 0, nvs = 0, nts = 0;
};

static void build_source_surface(SourceSurface& u, omg_geometry geo, const double* verts, int64_t nvs,
                                 const int64_t* tris, int64_t nts, int order, cudaStream_t s) {
    OMG_REQUIRE(verts && tris, "null source mesh");
    OMG_REQUIRE(nvs >= 3 && nts >= 1, "source mesh needs at least 3 vertices and 1 triangle");
    for (int64_t i = 0; i < 3 * nts; ++i)
        OMG_REQUIRE(tris[i] >= 0 && tris[i] < nvs, "source mesh triangle refers to a missing vertex");
    for (int64_t i = 0; i < 3 * nvs; ++i) OMG_REQUIRE(std::isfinite(verts[i]), "source mesh vertex not finite");
    const int64_t nv0 = geo ? geo->h.nv : 0, nt0 = geo ? geo->h.nt : 0;
    u.nv0 = nv0;
    u.nt0 = nt0;
    u.nvs = nvs;
    u.nts = nts;
    const int64_t nv = nv0 + nvs, nt = nt0 + nts;
    std::vector<double> V(3 * nv);
    std::vector<int32_t> T(3 * nt), tpos(nt, -1);
    if (geo) {
        std::copy(geo->h.V.begin(), geo->h.V.end(), V.begin());
        std::copy(geo->h.T.begin(), geo->h.T.end(), T.begin());
        for (int m = 0; m < geo->h.nmesh; ++m)
            for (int64_t t = geo->h.tbeg[m]; t < geo->h.tbeg[m + 1]; ++t)
                if (!geo->h.barrier[m]) tpos[t] = (int32_t)(geo->h.tidx[t] - geo->h.nvg);
    }
    std::copy(verts, verts + 3 * nvs, V.begin() + 3 * nv0);
    for (int64_t i = 0; i < 3 * nts; ++i) T[3 * nt0 + i] = (int32_t)(tris[i] + nv0);
    std::vector<int32_t> beg(nv + 1, 0), tri;
    std::vector<int8_t> loc;
    for (int64_t t = 0; t < nt; ++t)
        for (int j = 0; j < 3; ++j) beg[T[3 * t + j] + 1]++;
    for (int64_t v = 0; v < nv; ++v) beg[v + 1] += beg[v];
    tri.assign(beg[nv], 0);
    loc.assign(beg[nv], 0);
    std::vector<int32_t> fill(nv, 0);
    for (int64_t t = 0; t < nt; ++t)
        for (int j = 0; j < 3; ++j) {
            const int32_t v = T[3 * t + j];
            tri[beg[v] + fill[v]] = (int32_t)t;
            loc[beg[v] + fill[v]] = (int8_t)j;
            fill[v]++;
        }
    DevGeom& d = u.d;
    d.nv = nv;
    d.nt = nt;
    d.nP = geo ? geo->d.nP : 0;
    d.nPt = geo ? geo->d.nPt : 0;
    d.N = geo ? geo->d.N : 0;
    d.Nref = geo ? geo->d.Nref : 0;
    d.nmesh = (geo ? geo->h.nmesh : 0) + 1;
    d.V = upload(u.bufs, V, s);
    d.T = upload(u.bufs, T, s);
    d.tpos = upload(u.bufs, tpos, s);
    d.v2t_beg = upload(u.bufs, beg, s);
    d.v2t_tri = upload(u.bufs, tri, s);
    d.v2t_loc = upload(u.bufs, loc, s);
    u.bufs.emplace_back((size_t)nt * SREC * 8, s, true);
    d.srec = u.bufs.back().as<double>();
    u.bufs.emplace_back((size_t)nt * PREC * 8, s, true);
    d.prec = u.bufs.back().as<double>();
    u.bufs.emplace_back((size_t)nt * QREC * 8, s, true);
    d.qrec = u.bufs.back().as<double>();
    u.bufs.emplace_back(std::max<size_t>(1, tri.size()) * 3 * sizeof(double), s, true);
    d.v2t_q = u.bufs.back().as<double>();
    launch_prepare_triangles_order(d, order, s);
    launch_prepare_vertex_curls(d, s);
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char* omg_last_error(void) { return g_last_error.c_str(); }
const char* omg_version(void) { return "openmeeg_gb300 0.1 (sm_103a)"; }

int omg_context_create(int device, omg_context* out) {
    return guarded([&] {
        OMG_REQUIRE(out != nullptr, "null output handle");
        int n = 0;
        OMG_CUDA(cudaGetDeviceCount(&n));
        OMG_REQUIRE(device >= 0 && device < n, "no such CUDA device");
        auto ctx = std::make_unique<omg_context_s>();
        ctx->device = device;
        OMG_CUDA(cudaSetDevice(device));
        OMG_CUDA(cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking));
        ctx->stream = ctx->own;
        OMG_CUDA(cudaMalloc(&ctx->d_err, sizeof(int) * 4));
        OMG_CUDA(cudaMalloc(&ctx->d_errcol, sizeof(int64_t)));
        OMG_CUDA(cudaMalloc(&ctx->d_scalar, sizeof(double) * 4));
        OMG_CUDA(cudaMemset(ctx->d_err, 0, sizeof(int) * 4));
        // The temporaries of a call (head matrix, factor, digit planes: ~9 GB at N = 17926) are stream-ordered
        // allocations of the device's default pool; with its default release threshold of zero every
        // synchronization hands them back to the system and the next call maps them again (about 11 ms per
        // call at that size).  The pool keeps up to a quarter of the device's memory between calls; the rest
        // still goes back at each synchronization, and an allocation that fails trims the pool and retries.
        cudaMemPool_t pool;
        size_t fr = 0, tot = 0;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess && cudaMemGetInfo(&fr, &tot) == cudaSuccess) {
            uint64_t keep = 0;
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            keep = std::max<uint64_t>(keep, tot / 4);
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        ctx->launches_at_create = kernel_launch_count();
        *out = ctx.release();
    });
}

int omg_context_destroy(omg_context ctx) {
    return guarded([&] {
        if (!ctx) return;
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        ctx->stream = ctx->own;   // an external stream must not be used after its owner lets go
        release_context(ctx);
    });
}

int omg_context_set_stream(omg_context ctx, void* stream) {
    return guarded([&] {
        OMG_REQUIRE(ctx, "null context");
        ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
    });
}

int omg_context_synchronize(omg_context ctx) {
    return guarded([&] {
        OMG_REQUIRE(ctx, "null context");
        set_device(ctx);
        OMG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int omg_profile_enable(int32_t on) {
    return guarded([&] { profile_enable(on != 0); });
}

int omg_profile_read(int32_t max_entries, char* names, int64_t* launches, double* total_ms, int32_t* n_entries) {
    return guarded([&] {
        OMG_REQUIRE(max_entries >= 0 && n_entries, "bad arguments");
        auto v = profile_collect();
        int32_t n = 0;
        for (const auto& e : v) {
            if (n >= max_entries) break;
            if (names) {
                std::memset(names + 32 * n, 0, 32);
                std::strncpy(names + 32 * n, std::get<0>(e).c_str(), 31);
            }
            if (launches) launches[n] = std::get<1>(e);
            if (total_ms) total_ms[n] = std::get<2>(e);
            ++n;
        }
        *n_entries = n;
    });
}

int64_t omg_context_kernel_launches(omg_context ctx) {
    return ctx ? kernel_launch_count() - ctx->launches_at_create : 0;
}

static void finish_geometry(omg_context ctx, std::unique_ptr<omg_geometry_s>& g, omg_geometry* out) {
    g->ctx = ctx;
    upload_geometry(g.get());
    OMG_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->refs++;
    *out = g.release();
}

int omg_geometry_create(omg_context ctx, int32_t n_meshes, const int64_t* mesh_nverts, const double* verts,
                        const int64_t* mesh_ntris, const int64_t* tris, int32_t n_domains, const int32_t* dom_nbounds,
                        const int32_t* dom_bounds, const double* dom_sigma, omg_geometry* out) {
    return guarded([&] {
        OMG_REQUIRE(ctx && out && mesh_nverts && verts && mesh_ntris && tris && dom_nbounds && dom_bounds && dom_sigma,
                    "null argument");
        set_device(ctx);
        auto g = std::make_unique<omg_geometry_s>();
        g->h = build_geometry(n_meshes, mesh_nverts, verts, mesh_ntris, tris, n_domains, dom_nbounds, dom_bounds,
                              dom_sigma, {});
        finish_geometry(ctx, g, out);
    });
}

int omg_geometry_load(omg_context ctx, const char* geom_file, const char* cond_file, omg_geometry* out) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geom_file && cond_file && out, "null argument");
        set_device(ctx);
        auto g = std::make_unique<omg_geometry_s>();
        g->h = load_geometry_files(geom_file, cond_file);
        finish_geometry(ctx, g, out);
    });
}

int omg_geometry_destroy(omg_geometry geo) {
    return guarded([&] {
        if (!geo) return;
        cudaSetDevice(geo->ctx->device);
        cudaStreamSynchronize(geo->ctx->stream);
        release_geometry(geo);
    });
}

int omg_geometry_get_info(omg_geometry geo, omg_geometry_info* info) {
    return guarded([&] {
        OMG_REQUIRE(geo && info, "null argument");
        info->n_vertices = geo->h.nvg;
        info->n_triangles = geo->h.nt;
        info->n_unknowns = geo->h.N;
        info->n_triangle_unknowns = geo->h.nP;
        info->n_meshes = geo->h.nmesh;
        info->n_domains = (int32_t)geo->h.domains.size();
        info->n_mesh_pairs = (int32_t)geo->h.pairs.size();
        info->nested = geo->h.nested ? 1 : 0;
    });
}

int omg_geometry_set_conductivities(omg_geometry geo, const double* dom_sigma) {
    return guarded([&] {
        OMG_REQUIRE(geo && dom_sigma, "null argument");
        HostGeometry& h = geo->h;
        for (size_t d = 0; d < h.domains.size(); ++d) {
            OMG_REQUIRE(std::isfinite(dom_sigma[d]) && dom_sigma[d] >= 0.0, "conductivity must be finite and >= 0");
            OMG_REQUIRE((dom_sigma[d] == 0.0) == (h.domains[d].sigma == 0.0),
                        "a conductivity may not change to or from zero");
        }
        for (size_t d = 0; d < h.domains.size(); ++d) h.domains[d].sigma = dom_sigma[d];
        h.recompute_coefficients();
        geo->version++;
        std::vector<double> jump(h.nmesh);
        for (int m = 0; m < h.nmesh; ++m) jump[m] = h.conductivity_jump(m);
        cudaStream_t s = geo->ctx->stream;
        OMG_CUDA(cudaMemcpyAsync(geo->jump, jump.data(), jump.size() * 8, cudaMemcpyHostToDevice, s));
        std::vector<double> sig(h.domains.size());
        for (size_t d = 0; d < sig.size(); ++d) sig[d] = h.domains[d].sigma;
        OMG_CUDA(cudaMemcpyAsync(geo->dsigma, sig.data(), sig.size() * 8, cudaMemcpyHostToDevice, s));
        OMG_CUDA(cudaStreamSynchronize(s));
    });
}

int omg_headmat_dev(omg_context ctx, omg_geometry geo, const omg_integrator* integ, int32_t precision, double* hm,
                    int64_t ld) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && hm, "null argument");
        OMG_REQUIRE(ld >= geo->h.N, "ld must be >= N");
        OMG_REQUIRE(precision == OMG_PREC_FP64 || precision == OMG_PREC_MIXED, "unknown precision");
        set_device(ctx);
        reset_err(ctx);
        const omg_integrator it = integ ? *integ : default_hm_integrator();
        const int64_t N = geo->dg.N;
        DevBuf tmp = assemble_system(geo, it, precision, false);
        launch_symmetrize_to_reference(geo->dg, tmp.as<double>(), N, hm, ld, false, ctx->stream);
        check_err(ctx, "HeadMat");
    });
}

int omg_headmat_packed_dev(omg_context ctx, omg_geometry geo, const omg_integrator* integ, double* packed) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && packed, "null argument");
        set_device(ctx);
        reset_err(ctx);
        const omg_integrator it = integ ? *integ : default_hm_integrator();
        const int64_t N = geo->dg.N;
        DevBuf tmp = assemble_system(geo, it, OMG_PREC_FP64, false);
        launch_symmetrize_to_reference(geo->dg, tmp.as<double>(), N, packed, 0, true, ctx->stream);
        check_err(ctx, "HeadMat");
    });
}

int omg_dipsourcemat_dev(omg_context ctx, omg_geometry geo, const double* dipoles, int64_t n_dipoles,
                         const omg_integrator* integ, int32_t domain, double* dsm) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && (n_dipoles == 0 || (dipoles && dsm)), "null argument");
        OMG_REQUIRE(n_dipoles >= 0, "negative dipole count");
        set_device(ctx);
        reset_err(ctx);
        const omg_integrator it = integ ? *integ : default_dsm_integrator();
        dsm_internal(geo, dipoles, n_dipoles, it, domain, 0, dsm, geo->h.N);
        check_err(ctx, "DipSourceMat");
    });
}

int omg_head2eegmat_dev(omg_context ctx, omg_geometry geo, const double* electrodes, int64_t n_electrodes,
                        double* h2em, int64_t* sparse_cols, double* sparse_vals) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && (n_electrodes == 0 || electrodes), "null argument");
        OMG_REQUIRE(geo->n_eeg_cand > 0, "no interface touches a zero-conductivity domain");
        set_device(ctx);
        reset_err(ctx);
        if (h2em) OMG_CUDA(cudaMemsetAsync(h2em, 0, (size_t)n_electrodes * geo->h.N * 8, ctx->stream));
        launch_h2em(geo->d, electrodes, n_electrodes, geo->n_eeg_seg, geo->eeg_seg, geo->eeg_cand, 0, h2em,
                    n_electrodes, 1, 0,
                    sparse_cols, sparse_vals, ctx->stream);
        check_err(ctx, "Head2EEGMat");
    });
}

int omg_head2megmat_dev(omg_context ctx, omg_geometry geo, const double* squids, int64_t n_squids, double* h2mm) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && (n_squids == 0 || (squids && h2mm)), "null argument");
        set_device(ctx);
        reset_err(ctx);
        if (n_squids == 0) return;
        DevBuf F((size_t)n_squids * geo->h.nt * 8, ctx->stream);
        if (geo->h.shared) {   // on the vertex copies (internal numbering), then summed per distinct vertex
            const int64_t Nl = geo->d.N;
            DevBuf loc((size_t)Nl * n_squids * 8, ctx->stream);
            OMG_CUDA(cudaMemsetAsync(loc.p, 0, (size_t)Nl * n_squids * 8, ctx->stream));
            launch_h2mm(geo->d, squids, n_squids, geo->tmesh, geo->jump, 1, loc.as<double>(), 1, Nl, 0,
                        F.as<double>(), ctx->stream);
            launch_fold_to_reference(geo->h.N, geo->h.nvg, geo->d.nP, geo->gbeg, geo->gcopy, n_squids, loc.as<double>(),
                                     Nl, h2mm, n_squids, 1, ctx->stream);
        } else {
            OMG_CUDA(cudaMemsetAsync(h2mm, 0, (size_t)n_squids * geo->h.N * 8, ctx->stream));
            launch_h2mm(geo->d, squids, n_squids, geo->tmesh, geo->jump, 0, h2mm, n_squids, 1, 0, F.as<double>(),
                        ctx->stream);
        }
        check_err(ctx, "Head2MEGMat");
    });
}

int omg_dipsource2megmat_dev(omg_context ctx, const double* dipoles, int64_t n_dipoles, const double* squids,
                             int64_t n_squids, double* ds2mm) {
    return guarded([&] {
        OMG_REQUIRE(ctx && (n_dipoles == 0 || n_squids == 0 || (dipoles && squids && ds2mm)), "null argument");
        set_device(ctx);
        launch_ds2mm(dipoles, n_dipoles, squids, n_squids, ds2mm, n_squids, ctx->stream);
        OMG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

// SurfSourceMat (OpenMEEG/src/assembleSourceMat.cpp:22-64): for each boundary
// of the domain that holds the source surface, the N block (vertices of the
// boundary mesh x source vertices, coefficient +-K * orientation) and the D
// block (its triangles x source vertices, coefficient times -1/sigma).
int omg_surfsourcemat_dev(omg_context ctx, omg_geometry geo, const double* verts, int64_t n_verts,
                          const int64_t* tris, int64_t n_tris, const omg_integrator* integ, double* ssm) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && ssm, "null argument");
        set_device(ctx);
        const omg_integrator it = integ ? *integ : default_hm_integrator();
        check_integrator(it, false);
        cudaStream_t s = ctx->stream;
        reset_err(ctx);
        SourceSurface u;
        build_source_surface(u, geo, verts, n_verts, tris, n_tris, it.order, s);
        const HostGeometry& h = geo->h;
        // the domain of the source surface: every vertex must lie in the same one
        DevBuf sa((size_t)n_verts * h.nmesh * 8, s), dom((size_t)n_verts * sizeof(int), s);
        const double* pts = u.d.V + 3 * u.nv0;
        launch_mesh_solid_angles(pts, 3, n_verts, h.nmesh, geo->tbeg, geo->d.srec, sa.as<double>(), s);
        launch_domain_lookup(n_verts, h.nmesh, sa.as<double>(), geo->ndom, geo->maxb, geo->dnb, geo->bmesh,
                             geo->binside, geo->orient, geo->bgrp, -1, dom.as<int>(), ctx->d_err, s);
        std::vector<int> hdom(n_verts);
        OMG_CUDA(cudaMemcpyAsync(hdom.data(), dom.p, n_verts * sizeof(int), cudaMemcpyDeviceToHost, s));
        OMG_CUDA(cudaStreamSynchronize(s));
        const int d = hdom[0];
        OMG_REQUIRE(d >= 0, "the source mesh lies in no domain of the geometry");
        for (int v : hdom)
            OMG_REQUIRE(v == d, "the source mesh crosses an interface of the geometry (overlapping source mesh)");
        const double sigma = h.domains[d].sigma;
        OMG_REQUIRE(sigma != 0.0, "the source mesh lies in a zero-conductivity domain");
        const double L = -1.0 / sigma;
        const int64_t Nint = geo->d.N;
        DevBuf out((size_t)Nint * n_verts * 8, s);
        OMG_CUDA(cudaMemsetAsync(out.p, 0, (size_t)Nint * n_verts * 8, s));
        const int64_t tsb = u.nt0, tse = u.nt0 + n_tris, vsb = u.nv0, vse = u.nv0 + n_verts;
        for (const auto& b : h.domains[d].bounds) {
            const int m = b.mesh;
            const double coeffN = (b.inside ? kK : -kK) * b.o;
            const int64_t t1b = h.tbeg[m], t1e = h.tbeg[m + 1], n1 = t1e - t1b;
            {
                DevBuf S((size_t)n1 * n_tris * 8, s);   // unit-coefficient S block (the source is no unknown)
                launch_S_block(u.d, t1b, t1e, tsb, tse, false, 1.0, it.order, nullptr, 0, S.as<double>(),
                               ctx->d_err, s);
                launch_N_block(u.d, h.vbeg[m], h.vbeg[m + 1], t1b, t1e, vsb, vse, tsb, tse, false, coeffN, nullptr,
                               Nint, S.as<double>(), out.as<double>(), s, true, true);
            }
            if (!h.barrier[m]) {
                DevBuf D((size_t)n1 * n_tris * 24, s);
                launch_D_block(u.d, t1b, t1e, tsb, tse, it.order, D.as<double>(), ctx->d_err, s);
                launch_D_gather(u.d, t1b, t1e, tsb, tse, vsb, vse, coeffN * L, D.as<double>(), out.as<double>(), Nint,
                                s, true);
            }
        }
        if (h.shared)   // rows of the vertex copies summed per distinct vertex (a shared vertex gathers both meshes)
            launch_fold_to_reference(h.N, h.nvg, geo->d.nP, geo->gbeg, geo->gcopy, n_verts, out.as<double>(), Nint,
                                     ssm, 1, h.N, s);
        else
            launch_rows_to_reference(geo->d, n_verts, out.as<double>(), Nint, ssm, geo->d.Nref, s);
        check_err(ctx, "SurfSourceMat");
    });
}

// SurfSource2MEGMat (OpenMEEG/src/assembleSensors.cpp:102-125): the Ferguson
// field of the source surface's vertices at each sensor along its orientation.
int omg_surfsource2megmat_dev(omg_context ctx, const double* verts, int64_t n_verts, const int64_t* tris,
                              int64_t n_tris, const double* squids, int64_t n_squids, double* ss2mm) {
    return guarded([&] {
        OMG_REQUIRE(ctx && (n_squids == 0 || (squids && ss2mm)), "null argument");
        set_device(ctx);
        cudaStream_t s = ctx->stream;
        SourceSurface u;
        build_source_surface(u, nullptr, verts, n_verts, tris, n_tris, 3, s);
        if (n_squids > 0) {
            DevBuf F((size_t)n_squids * n_tris * 8, s);
            launch_h2mm(u.d, squids, n_squids, nullptr, nullptr, 0, ss2mm, n_squids, 1, 0, F.as<double>(), s, 1.0);
        }
        OMG_CUDA(cudaStreamSynchronize(s));
    });
}

// Domain of each point (Geometry::domain, geometry.cpp:146-154) and the
// output row of the points kept: those in a conducting domain, in input order
// (points in a zero-conductivity domain are dropped, assembleHeadMat.cpp:333-340).
struct KeptPoints {
    DevBuf dom, rows;
    int64_t kept = 0;
};
static void keep_conducting_points(KeptPoints& kp, omg_geometry geo, const double* pts, int64_t n, cudaStream_t s) {
    const HostGeometry& h = geo->h;
    kp.dom = DevBuf((size_t)std::max<int64_t>(n, 1) * sizeof(int), s);
    kp.rows = DevBuf((size_t)std::max<int64_t>(n, 1) * sizeof(int64_t), s);
    kp.kept = 0;
    if (n == 0) return;
    // FP32-screened solid angles: sums clear of the 2 pi boundary classify as in FP64, the rest are FP64 sums
    DevBuf sa((size_t)n * h.nmesh * 8, s);
    launch_mesh_solid_angles(pts, 3, n, h.nmesh, geo->tbeg, geo->d.srec, sa.as<double>(), s, true);
    launch_domain_lookup(n, h.nmesh, sa.as<double>(), geo->ndom, geo->maxb, geo->dnb, geo->bmesh, geo->binside,
                         geo->orient, geo->bgrp, -1, kp.dom.as<int>(), geo->ctx->d_err, s);
    check_err(geo->ctx, "point domain lookup");
    std::vector<int> hdom(n);
    OMG_CUDA(cudaMemcpyAsync(hdom.data(), kp.dom.p, n * sizeof(int), cudaMemcpyDeviceToHost, s));
    OMG_CUDA(cudaStreamSynchronize(s));
    std::vector<int64_t> rows(n);
    for (int64_t i = 0; i < n; ++i) {
        OMG_REQUIRE(hdom[i] >= 0, "a point lies in no domain of the geometry");
        rows[i] = h.domains[hdom[i]].sigma != 0.0 ? kp.kept++ : -1;
    }
    OMG_CUDA(cudaMemcpyAsync(kp.rows.p, rows.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    OMG_CUDA(cudaStreamSynchronize(s));   // the host vector goes out of scope
}

// Surf2VolMat (OpenMEEG/src/assembleHeadMat.cpp:325-363): potential at points
// inside the head from the surface unknowns; n_kept x Nref, column-major with
// leading dimension n_kept, columns in the reference numbering.
int omg_surf2volmat_dev(omg_context ctx, omg_geometry geo, const double* points, int64_t n_points, double* out,
                        int64_t* n_kept) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && n_kept && (n_points == 0 || (points && out)), "null argument");
        OMG_REQUIRE(n_points >= 0, "negative point count");
        set_device(ctx);
        cudaStream_t s = ctx->stream;
        reset_err(ctx);
        KeptPoints kp;
        keep_conducting_points(kp, geo, points, n_points, s);
        *n_kept = kp.kept;
        const int64_t ld = kp.kept, Nref = geo->d.Nref;
        if (kp.kept == 0) return;
        // meshes sharing vertices: the columns of every vertex copy first (nv + triangle unknowns), folded to the
        // distinct vertices afterwards (a shared vertex's P1 basis spans the triangles of all its meshes)
        const HostGeometry& h = geo->h;
        const int64_t ncol_w = h.shared ? h.nv + (Nref - h.nvg) : Nref, tshift = h.shared ? h.nv - h.nvg : 0;
        DevBuf work(h.shared ? (size_t)ld * ncol_w * 8 : 0, s);
        double* dst = h.shared ? work.as<double>() : out;
        OMG_CUDA(cudaMemsetAsync(dst, 0, (size_t)ld * ncol_w * 8, s));
        // chunk the points so the P1 scratch stays near 512 MB
        const int64_t per = std::max<int64_t>(1, std::min<int64_t>(4096, (512ll << 20) / (geo->h.nt * 24)));
        DevBuf p1((size_t)std::min(per, n_points) * geo->h.nt * 24, s);
        for (int64_t p0 = 0; p0 < n_points; p0 += per)
            launch_partial_block(geo->d, p0, std::min(per, n_points - p0), points, kp.dom.as<int>(),
                                 kp.rows.as<int64_t>(), geo->tmesh, geo->tidx_ref, geo->barrier, geo->orient,
                                 geo->maxb, geo->dnb, geo->bmesh, geo->binside, geo->dsigma, p1.as<double>(), dst, ld,
                                 s, tshift);
        if (h.shared) launch_fold_columns(ld, Nref, h.nvg, h.nv, geo->gbeg, geo->gcopy, dst, ld, out, ld, s);
        check_err(ctx, "Surf2VolMat");
    });
}

// DipSource2InternalPotMat (OpenMEEG/src/assembleSourceMat.cpp:154-187):
// n_kept x n_dipoles, column-major with leading dimension n_kept.  domain >= 0
// places every dipole in that domain (the reference's domain_name argument).
int omg_dipsource2internalpotmat_dev(omg_context ctx, omg_geometry geo, const double* dipoles, int64_t n_dipoles,
                                     const double* points, int64_t n_points, int32_t domain, double* out,
                                     int64_t* n_kept) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && n_kept && (n_points == 0 || points) && (n_dipoles == 0 || dipoles),
                    "null argument");
        OMG_REQUIRE(n_points >= 0 && n_dipoles >= 0, "negative size");
        OMG_REQUIRE(domain >= -1 && domain < geo->ndom, "domain index out of range");
        set_device(ctx);
        cudaStream_t s = ctx->stream;
        reset_err(ctx);
        KeptPoints kp;
        keep_conducting_points(kp, geo, points, n_points, s);
        *n_kept = kp.kept;
        if (kp.kept == 0 || n_dipoles == 0) return;
        OMG_REQUIRE(out, "null argument");
        const HostGeometry& h = geo->h;
        DevBuf sa((size_t)n_dipoles * h.nmesh * 8, s), ddom((size_t)n_dipoles * sizeof(int), s);
        if (domain < 0)
            launch_mesh_solid_angles(dipoles, 6, n_dipoles, h.nmesh, geo->tbeg, geo->d.srec, sa.as<double>(), s,
                                     true);
        launch_domain_lookup(n_dipoles, h.nmesh, sa.as<double>(), geo->ndom, geo->maxb, geo->dnb, geo->bmesh,
                             geo->binside, geo->orient, geo->bgrp, domain, ddom.as<int>(), ctx->d_err, s);
        launch_dipole_internal_pot(points, kp.dom.as<int>(), kp.rows.as<int64_t>(), n_points, dipoles, ddom.as<int>(),
                                   n_dipoles, geo->dsigma, out, kp.kept, s);
        check_err(ctx, "DipSource2InternalPotMat");
    });
}

// Injection triangles of EIT electrodes (Sensors::findInjectionTriangles,
// sensors.cpp:167-215): the nearest triangle of the interfaces touching a
// zero-conductivity domain, and for an electrode of radius r > 0 whose nearest
// triangle is smaller than 4 pi r^2, a depth-first walk over neighbouring
// triangles whose centres lie within r.  The walk follows the first three
// entries of Mesh::adjacent_triangles (mesh.h:164-172): the triangles met twice
// while scanning the incidence lists (triangle order) of the triangle's
// vertices -- which include the triangle itself, so one edge neighbour is
// left out, as in the reference.  Weight pi r^2 / (area of the triangles)
// for r > 0; 1 / area for a point electrode (assembleSourceMat.cpp:141-150).
struct Injection {
    std::vector<int64_t> tri;
    std::vector<double> coef;
};
static std::vector<Injection> injection_triangles(const HostGeometry& h, const std::vector<double>& pos,
                                                  const std::vector<double>& radii,
                                                  const std::vector<int64_t>& nearest) {
    const double pi = 3.14159265358979323846;
    auto vtx = [&](int64_t v) { return &h.V[3 * v]; };
    auto area = [&](int64_t t) {
        const double *a = vtx(h.T[3 * t]), *b = vtx(h.T[3 * t + 1]), *c = vtx(h.T[3 * t + 2]);
        const double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, w[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        const double n[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
        return std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]) / 2.0;
    };
    auto mesh_of = [&](int64_t t) {
        return (int)(std::upper_bound(h.tbeg.begin(), h.tbeg.end(), t) - h.tbeg.begin()) - 1;
    };
    auto adjacent = [&](int64_t t) {
        const int m = mesh_of(t);
        std::vector<std::pair<int64_t, int>> cnt;
        std::vector<int64_t> res;
        for (int j = 0; j < 3; ++j) {
            const int64_t v = h.T[3 * t + j];
            for (int q = h.v2t_beg[v]; q < h.v2t_beg[v + 1]; ++q) {
                const int64_t t2 = h.v2t_tri[q];
                if (t2 < h.tbeg[m] || t2 >= h.tbeg[m + 1]) continue;
                auto it = std::find_if(cnt.begin(), cnt.end(), [&](const auto& c) { return c.first == t2; });
                if (it == cnt.end()) {
                    cnt.push_back({t2, 1});
                } else if (++it->second == 2) {
                    res.push_back(t2);
                }
            }
        }
        return res;
    };
    const size_t ne = nearest.size();
    std::vector<Injection> out(ne);
    for (size_t e = 0; e < ne; ++e) {
        const int64_t t0 = nearest[e];
        OMG_REQUIRE(t0 >= 0, "no interface touches a zero-conductivity domain");
        const double r = radii[e];
        const bool point = std::fabs(r) < 2.2250738585072014e-308;   // almost_equal(radius, 0.0)
        std::vector<int64_t> tris{t0};
        if (!point && area(t0) < 4 * pi * r * r) {
            std::vector<int64_t> seen{t0}, stack{t0};
            while (!stack.empty()) {
                const int64_t t = stack.back();
                stack.pop_back();
                const double *a = vtx(h.T[3 * t]), *b = vtx(h.T[3 * t + 1]), *c = vtx(h.T[3 * t + 2]);
                const double d[3] = {(a[0] + b[0] + c[0]) / 3.0 - pos[3 * e], (a[1] + b[1] + c[1]) / 3.0 - pos[3 * e + 1],
                                     (a[2] + b[2] + c[2]) / 3.0 - pos[3 * e + 2]};
                if (std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) < r) {
                    if (t != t0) tris.push_back(t);
                    const std::vector<int64_t> adj = adjacent(t);
                    for (size_t i = 0; i < std::min<size_t>(3, adj.size()); ++i)
                        if (std::find(seen.begin(), seen.end(), adj[i]) == seen.end()) {
                            seen.push_back(adj[i]);
                            stack.push_back(adj[i]);
                        }
                }
            }
        }
        out[e].tri = tris;
        if (point) {
            for (int64_t t : tris) out[e].coef.push_back(1.0 / area(t));
        } else {
            double tot = 0.0;
            for (int64_t t : tris) tot += area(t);
            out[e].coef.assign(tris.size(), pi * r * r / tot);
        }
    }
    return out;
}

// EITSourceMat (OpenMEEG/src/assembleSourceMat.cpp:109-152): Nref x n_electrodes,
// column-major; only the transfer-matrix rows of the injection triangles are formed.
int omg_eitsourcemat_dev(omg_context ctx, omg_geometry geo, const double* positions, const double* radii,
                         int64_t n_electrodes, const omg_integrator* integ, double* out) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && (n_electrodes == 0 || (positions && out)), "null argument");
        OMG_REQUIRE(n_electrodes >= 0, "negative electrode count");
        set_device(ctx);
        const omg_integrator it = integ ? *integ : default_hm_integrator();
        check_integrator(it, false);
        cudaStream_t s = ctx->stream;
        reset_err(ctx);
        const HostGeometry& h = geo->h;
        const int64_t Nref = geo->d.Nref, ne = n_electrodes;
        if (ne == 0) return;
        OMG_REQUIRE(geo->n_eeg_cand > 0, "no interface touches a zero-conductivity domain");
        ensure_order(geo, it.order);
        std::vector<double> hpos(3 * ne), hrad(ne, 0.0);
        OMG_CUDA(cudaMemcpyAsync(hpos.data(), positions, 3 * ne * 8, cudaMemcpyDeviceToHost, s));
        if (radii) OMG_CUDA(cudaMemcpyAsync(hrad.data(), radii, ne * 8, cudaMemcpyDeviceToHost, s));
        DevBuf near((size_t)ne * 8, s);
        launch_nearest_triangle(geo->d, positions, ne, geo->n_eeg_cand, geo->eeg_cand, near.as<int64_t>(), s);
        std::vector<int64_t> hnear(ne);
        OMG_CUDA(cudaMemcpyAsync(hnear.data(), near.p, ne * 8, cudaMemcpyDeviceToHost, s));
        OMG_CUDA(cudaStreamSynchronize(s));
        const std::vector<Injection> inj = injection_triangles(h, hpos, hrad, hnear);
        // distinct injection triangles, grouped by mesh (ids are positions in `uniq`)
        std::vector<int64_t> uniq;
        for (const auto& e : inj) uniq.insert(uniq.end(), e.tri.begin(), e.tri.end());
        std::sort(uniq.begin(), uniq.end());
        uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
        std::vector<int64_t> ebeg{0}, eid;
        std::vector<double> ecoef;
        for (const auto& e : inj) {
            for (size_t q = 0; q < e.tri.size(); ++q) {
                eid.push_back(std::lower_bound(uniq.begin(), uniq.end(), e.tri[q]) - uniq.begin());
                ecoef.push_back(e.coef[q]);
            }
            ebeg.push_back((int64_t)eid.size());
        }
        DevBuf d_uniq(uniq.size() * 8, s), d_ebeg(ebeg.size() * 8, s), d_eid(eid.size() * 8, s),
            d_ecoef(ecoef.size() * 8, s);
        OMG_CUDA(cudaMemcpyAsync(d_uniq.p, uniq.data(), uniq.size() * 8, cudaMemcpyHostToDevice, s));
        OMG_CUDA(cudaMemcpyAsync(d_ebeg.p, ebeg.data(), ebeg.size() * 8, cudaMemcpyHostToDevice, s));
        OMG_CUDA(cudaMemcpyAsync(d_eid.p, eid.data(), eid.size() * 8, cudaMemcpyHostToDevice, s));
        OMG_CUDA(cudaMemcpyAsync(d_ecoef.p, ecoef.data(), ecoef.size() * 8, cudaMemcpyHostToDevice, s));
        OMG_CUDA(cudaMemsetAsync(out, 0, (size_t)Nref * ne * 8, s));
        int64_t ntmax = 1;
        for (int m = 0; m < h.nmesh; ++m) ntmax = std::max<int64_t>(ntmax, h.tbeg[m + 1] - h.tbeg[m]);
        const int64_t per = std::max<int64_t>(
            1, std::min<int64_t>({4096, (256ll << 20) / (Nref * 8), (512ll << 20) / (ntmax * 24)}));
        const int64_t nu = (int64_t)uniq.size();
        DevBuf R((size_t)std::min(per, nu) * Nref * 8, s), tmp((size_t)std::min(per, nu) * ntmax * 24, s);
        for (int m = 0; m < h.nmesh; ++m) {
            if (!h.barrier[m]) continue;   // rows of non-barrier triangles are never filled
            const int64_t ub = std::lower_bound(uniq.begin(), uniq.end(), h.tbeg[m]) - uniq.begin();
            const int64_t ue = std::lower_bound(uniq.begin(), uniq.end(), h.tbeg[m + 1]) - uniq.begin();
            for (int64_t k0 = ub; k0 < ue; k0 += per) {
                const int64_t nk = std::min(per, ue - k0);
                OMG_CUDA(cudaMemsetAsync(R.p, 0, (size_t)nk * Nref * 8, s));
                for (const auto& p : h.pairs) {
                    if (p.m1 != m) continue;
                    const int m2 = p.m2;
                    const bool self = (m2 == m);
                    launch_eit_rows(geo->d, d_uniq.as<int64_t>() + k0, nk, h.tbeg[m2], h.tbeg[m2 + 1], h.vbeg[m2],
                                    h.vbeg[m2 + 1], self, !self && !h.barrier[m2], kK * p.orientation, -p.cS,
                                    geo->tidx_ref, it.order, tmp.as<double>(), R.as<double>(), s);
                }
                launch_eit_combine(Nref, ne, d_ebeg.as<int64_t>(), d_eid.as<int64_t>(), d_ecoef.as<double>(), k0, nk,
                                   R.as<double>(), out, s);
            }
        }
        check_err(ctx, "EITSourceMat");
    });
}

int omg_geometry_get_layout(omg_geometry geo, int32_t max_meshes, omg_mesh_layout* out) {
    return guarded([&] {
        OMG_REQUIRE(geo && out, "null argument");
        const HostGeometry& h = geo->h;
        OMG_REQUIRE(max_meshes >= h.nmesh, "output too small");
        require_distinct_vertices(geo, "the mesh layout");
        for (int m = 0; m < h.nmesh; ++m) {
            omg_mesh_layout& L = out[m];
            L.vbeg = h.vbeg[m];
            L.vend = h.vbeg[m + 1];
            L.tri_unknown = h.barrier[m] ? -1 : h.tidx[h.tbeg[m]];
            L.n_triangles = h.tbeg[m + 1] - h.tbeg[m];
            L.barrier = h.barrier[m];
            L.orientation = h.orient[m];
            L.outermost = h.outermost[m];
            L.reserved = 0;
        }
    });
}

int omg_geometry_get_pairs(omg_geometry geo, int32_t max_pairs, omg_mesh_pair* out, int32_t* n_pairs) {
    return guarded([&] {
        OMG_REQUIRE(geo && n_pairs, "null argument");
        const auto& P = geo->h.pairs;
        *n_pairs = (int32_t)P.size();
        if (!out) return;
        OMG_REQUIRE(max_pairs >= (int32_t)P.size(), "output too small");
        for (size_t k = 0; k < P.size(); ++k) out[k] = {P[k].m1, P[k].m2, P[k].orientation, 0, P[k].cS, P[k].cN, P[k].cD};
    });
}

int omg_dipole_domains_dev(omg_context ctx, omg_geometry geo, const double* dipoles, int64_t n_dipoles,
                           int32_t* domains) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && (n_dipoles == 0 || (dipoles && domains)), "null argument");
        set_device(ctx);
        reset_err(ctx);
        if (n_dipoles == 0) return;
        cudaStream_t s = ctx->stream;
        DevBuf sa((size_t)n_dipoles * geo->h.nmesh * 8, s);
        launch_mesh_solid_angles(dipoles, 6, n_dipoles, geo->h.nmesh, geo->tbeg, geo->d.srec, sa.as<double>(), s);
        launch_domain_lookup(n_dipoles, geo->h.nmesh, sa.as<double>(), geo->ndom, geo->maxb, geo->dnb, geo->bmesh,
                             geo->binside, geo->orient, geo->bgrp, -1, domains, ctx->d_err, s);
        OMG_CUDA(cudaStreamSynchronize(s));
    });
}

int omg_head2megmat_mesh_dev(omg_context ctx, omg_geometry geo, const double* squids, int64_t n_squids, int32_t mesh,
                             double* out) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && (n_squids == 0 || (squids && out)), "null argument");
        require_distinct_vertices(geo, "the per-mesh Head2MEGMat");
        OMG_REQUIRE(mesh >= 0 && mesh < geo->h.nmesh, "mesh index out of range");
        set_device(ctx);
        reset_err(ctx);
        if (n_squids == 0) return;
        cudaStream_t s = ctx->stream;
        std::vector<double> unit(geo->h.nmesh, 0.0);
        unit[mesh] = 1.0;
        DevBuf jump(unit.size() * 8, s), F((size_t)n_squids * geo->h.nt * 8, s);
        OMG_CUDA(cudaMemcpyAsync(jump.p, unit.data(), unit.size() * 8, cudaMemcpyHostToDevice, s));
        OMG_CUDA(cudaMemsetAsync(out, 0, (size_t)n_squids * geo->h.N * 8, s));
        launch_h2mm(geo->d, squids, n_squids, geo->tmesh, jump.as<double>(), 0, out, n_squids, 1, 0, F.as<double>(), s);
        check_err(ctx, "Head2MEGMat (one mesh)");
    });
}

int omg_dipsourcemat_vjp_dev(omg_context ctx, omg_geometry geo, const double* dipoles, int64_t n_dipoles,
                             const omg_integrator* integ, int32_t domain, const double* U, int64_t ldu, double* out) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && (n_dipoles == 0 || (dipoles && U && out)), "null argument");
        require_distinct_vertices(geo, "the DipSourceMat vector-Jacobian product");
        OMG_REQUIRE(ldu >= geo->h.N, "ldu must be >= N");
        OMG_REQUIRE(domain >= -1 && domain < geo->ndom, "domain index out of range");
        set_device(ctx);
        reset_err(ctx);
        if (n_dipoles == 0) return;
        const omg_integrator it = integ ? *integ : default_dsm_integrator();
        check_integrator(it, true);
        cudaStream_t s = ctx->stream;
        DevBuf sa((size_t)n_dipoles * geo->h.nmesh * 8, s), dom((size_t)n_dipoles * sizeof(int), s);
        launch_mesh_solid_angles(dipoles, 6, n_dipoles, geo->h.nmesh, geo->tbeg, geo->d.srec, sa.as<double>(), s);
        launch_domain_lookup(n_dipoles, geo->h.nmesh, sa.as<double>(), geo->ndom, geo->maxb, geo->dnb, geo->bmesh,
                             geo->binside, geo->orient, geo->bgrp, domain, dom.as<int>(), ctx->d_err, s);
        const int64_t per = std::max<int64_t>(1, std::min<int64_t>(4096, (512ll << 20) / (geo->h.nt * 48)));
        DevBuf part((size_t)std::min(per, n_dipoles) * geo->h.nt * 48, s);
        for (int64_t d0 = 0; d0 < n_dipoles; d0 += per) {
            const int64_t n = std::min(per, n_dipoles - d0);
            launch_dsm_vjp(geo->d, d0, n, dipoles, geo->tmesh, geo->tidx_ref, geo->barrier, geo->orient, dom.as<int>(),
                           geo->maxb, geo->dnb, geo->bmesh, geo->binside, geo->dsigma, it.order, it.levels, it.tol, U,
                           ldu, part.as<double>(), out, s);
        }
        check_err(ctx, "DipSourceMat vjp");
    });
}

int omg_gemm_f64_dev(omg_context ctx, int32_t trans_a, int32_t trans_b, int64_t m, int64_t n, int64_t k, double alpha,
                     const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc) {
    return guarded([&] {
        OMG_REQUIRE(ctx && (m == 0 || n == 0 || (A && B && C)), "null argument");
        set_device(ctx);
        if (k == 0) {
            OMG_REQUIRE(beta == 0.0 || beta == 1.0, "k = 0 with a general beta is not supported");
            if (beta == 0.0)
                for (int64_t j = 0; j < n; ++j) OMG_CUDA(cudaMemsetAsync(C + j * ldc, 0, (size_t)m * 8, ctx->stream));
        } else {
            gemm<double>(m, n, k, alpha, A, lda, trans_a != 0, B, ldb, trans_b != 0, beta, C, ldc, ctx->stream);
        }
        OMG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int omg_solver_create(omg_context ctx, omg_geometry geo, const omg_integrator* integ, int32_t precision,
                      omg_solver* out) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && out, "null argument");
        OMG_REQUIRE(precision == OMG_PREC_FP64 || precision == OMG_PREC_MIXED, "unknown precision");
        set_device(ctx);
        reset_err(ctx);
        auto sv = std::make_unique<omg_solver_s>();
        sv->ctx = ctx;
        sv->geo = geo;
        sv->precision = precision;
        sv->N = geo->dg.N;
        sv->nP = geo->d.nP;
        sv->persistent = true;
        const omg_integrator it = integ ? *integ : default_hm_integrator();
        DevBuf hm = assemble_system(geo, it, precision, true);
        check_err(ctx, "HeadMat");
        sv->rebuild = [geo, it, precision] { return assemble_system(geo, it, precision, true); };
        solver_factor_or_pivot(sv.get(), std::move(hm), sv->rebuild);
        ctx->refs++;
        geo->refs++;
        *out = sv.release();
    });
}

int omg_solver_from_headmat_dev(omg_context ctx, omg_geometry geo, const double* hm, int64_t ld, int32_t precision,
                                omg_solver* out) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo && hm && out, "null argument");
        OMG_REQUIRE(ld >= geo->h.N, "ld must be >= N");
        set_device(ctx);
        reset_err(ctx);
        auto sv = std::make_unique<omg_solver_s>();
        sv->ctx = ctx;
        sv->geo = geo;
        sv->precision = precision;
        sv->N = geo->dg.N;
        sv->nP = geo->d.nP;
        sv->persistent = true;
        auto copy_in = [&] {
            DevBuf A((size_t)sv->N * sv->N * 8, ctx->stream, true);
            launch_from_reference_dense(geo->dg, hm, ld, A.as<double>(), sv->N, ctx->stream);
            return A;
        };
        // (the caller's matrix is not kept: a stalled refinement is reported, not re-solved)
        solver_factor_or_pivot(sv.get(), copy_in(), copy_in);
        ctx->refs++;
        geo->refs++;
        *out = sv.release();
    });
}

int omg_solver_solve_dev(omg_solver sv, double* b, int64_t ldb, int64_t nrhs) {
    return guarded([&] {
        OMG_REQUIRE(sv && b, "null argument");
        OMG_REQUIRE(ldb >= sv->geo->h.N && nrhs >= 0, "bad right-hand side shape");
        set_device(sv->ctx);
        cudaStream_t s = sv->ctx->stream;
        const int64_t N = sv->N, nv = sv->geo->h.nvg, nP = sv->nP, nPt = sv->geo->d.nPt;
        // reference -> internal numbering: triangle rows [nv, nv+nPt) first, zero padding, then vertices [0, nv)
        DevBuf X((size_t)N * nrhs * 8, s);
        double* x = X.as<double>();
        OMG_CUDA(cudaMemsetAsync(x, 0, (size_t)N * nrhs * 8, s));
        for (int64_t j = 0; j < nrhs; ++j) {
            OMG_CUDA(cudaMemcpyAsync(x + j * N, b + j * ldb + nv, (size_t)nPt * 8, cudaMemcpyDeviceToDevice, s));
            OMG_CUDA(cudaMemcpyAsync(x + j * N + nP, b + j * ldb, (size_t)nv * 8, cudaMemcpyDeviceToDevice, s));
        }
        solver_solve_internal(sv, x, N, nrhs);
        for (int64_t j = 0; j < nrhs; ++j) {
            OMG_CUDA(cudaMemcpyAsync(b + j * ldb + nv, x + j * N, (size_t)nPt * 8, cudaMemcpyDeviceToDevice, s));
            OMG_CUDA(cudaMemcpyAsync(b + j * ldb, x + j * N + nP, (size_t)nv * 8, cudaMemcpyDeviceToDevice, s));
        }
        OMG_CUDA(cudaStreamSynchronize(s));
    });
}

int omg_solver_set_refinement(omg_solver sv, double tol, int32_t max_steps) {
    return guarded([&] {
        OMG_REQUIRE(sv, "null argument");
        OMG_REQUIRE(tol > 0.0 && max_steps >= 0, "bad refinement controls");
        sv->refine_tol = tol;
        sv->max_refine = max_steps;
    });
}

int omg_solver_destroy(omg_solver sv) {
    return guarded([&] {
        if (!sv) return;
        cudaSetDevice(sv->ctx->device);
        cudaStreamSynchronize(sv->ctx->stream);
        omg_context ctx = sv->ctx;
        omg_geometry geo = sv->geo;
        delete sv;
        release_geometry(geo);
        release_context(ctx);
    });
}

// Adjoint gain (gain.h:78-136): factor once, solve the sensor rows, contract
// with the DipSourceMat.
static void gain_pipeline(omg_context ctx, omg_geometry geo, int precision, const omg_integrator& hm_it,
                          const omg_integrator& dsm_it, const double* dip, int64_t nd, const double* el, int64_t ne,
                          const double* sq, int64_t nm, double* geeg, double* gmeg, omg_gain_stats* st) {
    cudaStream_t s = ctx->stream;
    const int64_t N = geo->dg.N, k = ne + nm;
    cudaEvent_t ev[7], ev_src;
    for (auto& e : ev) OMG_CUDA(cudaEventCreate(&e));
    OMG_CUDA(cudaEventCreateWithFlags(&ev_src, cudaEventDisableTiming));
    OMG_CUDA(cudaEventRecord(ev[0], s));
    reset_err(ctx);
    const int64_t live0 = g_dev_live.load();
    g_dev_peak.store(live0);
    auto sv = std::make_unique<omg_solver_s>();
    sv->ctx = ctx;
    sv->geo = geo;
    sv->precision = precision;
    sv->N = N;
    sv->nP = geo->d.nP;
    // right-hand sides (internal numbering) and DSM: allocated on the main stream, which uses them last
    DevBuf B((size_t)N * std::max<int64_t>(k, 1) * 8, s), DSM((size_t)N * std::max<int64_t>(nd, 1) * 8, s);
    DevBuf F((size_t)std::max<int64_t>(nm, 1) * geo->h.nt * 8, s);
    OMG_CUDA(cudaMemsetAsync(B.p, 0, (size_t)N * std::max<int64_t>(k, 1) * 8, s));
    if (precision == OMG_PREC_MIXED) ensure_gg_tables(geo);
    // The sources do not depend on the head matrix.  The sensor right-hand sides are enqueued first on the
    // second stream (joined before the solves); the DipSourceMat and DipSource2MEGMat go to the second stream
    // after the factorization and run under the latency-bound chains of the FP32 solves, which leave most SMs
    // idle (joined before the contraction).
    ensure_aux(ctx);
    cudaStream_t s2 = ctx->aux;
    OMG_CUDA(cudaEventRecord(ev[5], s));
    OMG_CUDA(cudaStreamWaitEvent(s2, ev[5], 0));
    DevBuf dom;
    {
        StreamSwap on_aux(ctx, s2);   // the library calls below take the context's stream
        if (ne > 0) {
            OMG_REQUIRE(geo->n_eeg_cand > 0, "no interface touches a zero-conductivity domain");
            launch_h2em(geo->d, el, ne, geo->n_eeg_seg, geo->eeg_seg, geo->eeg_cand, 1, B.as<double>(), 1, N, 0,
                        nullptr, nullptr, s2);
        }
        if (nm > 0 && geo->h.shared) {   // on the vertex copies, then summed per distinct vertex
            const int64_t Nl = geo->d.N;
            DevBuf loc((size_t)Nl * nm * 8, s2);
            OMG_CUDA(cudaMemsetAsync(loc.p, 0, (size_t)Nl * nm * 8, s2));
            launch_h2mm(geo->d, sq, nm, geo->tmesh, geo->jump, 1, loc.as<double>(), 1, Nl, 0, F.as<double>(), s2);
            launch_fold_rows(N, geo->d.nP, geo->gbeg, geo->gcopy, nm, loc.as<double>(), Nl, B.as<double>() + ne * N,
                             N, s2);
        } else if (nm > 0) {
            launch_h2mm(geo->d, sq, nm, geo->tmesh, geo->jump, 1, B.as<double>(), 1, N, ne, F.as<double>(), s2);
        }
        OMG_CUDA(cudaEventRecord(ev[6], s2));
    }
    DevBuf hm = assemble_system(geo, hm_it, precision, false);
    OMG_CUDA(cudaEventRecord(ev[1], s));
    OMG_CUDA(cudaStreamWaitEvent(s, ev[6], 0));
    OMG_CUDA(cudaEventRecord(ev[2], s));
    sv->rebuild = [geo, hm_it, precision] { return assemble_system(geo, hm_it, precision, false); };
    // the sources run beside the solves: the sweeps take five eighths of the SMs (config1, solves +
    // sources: 96 CTAs 12.2 ms, 152 CTAs 12.6 ms, 64 CTAs 12.3 ms, 48 CTAs 13.8 ms)
    sv->sweep_ctas = std::max(1, n_sm() * 5 / 8);
    solver_factor_or_pivot(sv.get(), std::move(hm), sv->rebuild);
    OMG_CUDA(cudaEventRecord(ev[3], s));
    {   // after the factorization's last work on the second stream (stream order); every stage of the
        // pipeline is throughput-bound, so the sources run where they take the least (under the assembly
        // they slowed the FP64-bound near-pair kernel by more than they saved later)
        StreamSwap on_aux(ctx, s2);
        dsm_internal(geo, dip, nd, dsm_it, -1, 1, DSM.as<double>(), N, precision, nullptr, 0, &dom);
        if (nm > 0) launch_ds2mm(dip, nd, sq, nm, gmeg, nm, s2);
        OMG_CUDA(cudaEventRecord(ev_src, s2));
    }
    {   // the solves on the highest-priority stream, ordered after the main stream's work and back
        OMG_CUDA(cudaEventRecord(ev[5], s));
        OMG_CUDA(cudaStreamWaitEvent(ctx->hi, ev[5], 0));
        {
            StreamSwap on_hi(ctx, ctx->hi);
            solver_solve_internal(sv.get(), B.as<double>(), N, k);
            OMG_CUDA(cudaEventRecord(ev[5], ctx->hi));
        }
        OMG_CUDA(cudaStreamWaitEvent(s, ev[5], 0));
    }
    OMG_CUDA(cudaStreamWaitEvent(s, ev_src, 0));
    // the factor is not needed past the solves: its memory (the FP32 factor, its copies and the digit planes,
    // most of the device at the largest heads) is returned before the contraction allocates its digits
    const int sv_steps = sv->last_steps;
    const double sv_residual = sv->last_residual;
    const bool sv_tc = sv->tc_residual;
    sv.reset();
    // G = Y^T DSM over the rows where DSM can be nonzero (the source meshes' triangles and vertices)
    std::vector<int> hdom(nd);
    if (nd > 0) {
        OMG_CUDA(cudaMemcpyAsync(hdom.data(), dom.p, nd * sizeof(int), cudaMemcpyDeviceToHost, s));
        OMG_CUDA(cudaStreamSynchronize(s));
    }
    gain_contract(gain_row_ranges(geo, meshes_of_domains(geo, hdom)), B.as<double>(), N, ne, nm, DSM.as<double>(), nd,
                  geeg, gmeg, s, precision, ctx->d_err);
    OMG_CUDA(cudaEventRecord(ev[4], s));
    check_err(ctx, "gain");
    if (st) {
        float a = 0, b = 0, c = 0, d = 0;
        OMG_CUDA(cudaEventElapsedTime(&a, ev[0], ev[1]));
        OMG_CUDA(cudaEventElapsedTime(&b, ev[1], ev[2]));
        OMG_CUDA(cudaEventElapsedTime(&c, ev[2], ev[3]));
        OMG_CUDA(cudaEventElapsedTime(&d, ev[3], ev[4]));
        st->t_headmat_ms = a;
        st->t_sources_ms = b;
        st->t_factor_ms = c;
        st->t_solve_ms = d;
        st->t_total_ms = a + b + c + d;
        st->refinement_steps = sv_steps;
        st->residual_mode = precision == OMG_PREC_FP64 ? 0 : (sv_tc ? 1 : 2);
        st->final_residual = sv_residual;
        st->device_bytes = g_dev_peak.load() - live0;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    cudaEventDestroy(ev_src);
}

int omg_gain_dev(omg_context ctx, omg_geometry geo, int32_t precision, const omg_integrator* hm_integ,
                 const omg_integrator* dsm_integ, const double* dipoles, int64_t n_dipoles, const double* electrodes,
                 int64_t n_electrodes, const double* squids, int64_t n_squids, double* gain_eeg, double* gain_meg,
                 omg_gain_stats* stats) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo, "null argument");
        OMG_REQUIRE(precision == OMG_PREC_FP64 || precision == OMG_PREC_MIXED, "unknown precision");
        OMG_REQUIRE(n_dipoles >= 0 && n_electrodes >= 0 && n_squids >= 0, "negative count");
        OMG_REQUIRE(n_dipoles == 0 || dipoles, "null dipoles");
        OMG_REQUIRE(n_electrodes == 0 || (electrodes && (gain_eeg || n_dipoles == 0)), "null electrodes or EEG output");
        OMG_REQUIRE(n_squids == 0 || (squids && (gain_meg || n_dipoles == 0)), "null squids or MEG output");
        set_device(ctx);
        const omg_integrator hi = hm_integ ? *hm_integ : default_hm_integrator();
        const omg_integrator di = dsm_integ ? *dsm_integ : default_dsm_integrator();
        gain_pipeline(ctx, geo, precision, hi, di, dipoles, n_dipoles, electrodes, n_electrodes, squids, n_squids,
                      gain_eeg, gain_meg, stats);
    });
}

int omg_gain_host(omg_context ctx, omg_geometry geo, int32_t precision, const omg_integrator* hm_integ,
                  const omg_integrator* dsm_integ, const double* dipoles, int64_t n_dipoles, const double* electrodes,
                  int64_t n_electrodes, const double* squids, int64_t n_squids, double* gain_eeg, double* gain_meg,
                  omg_gain_stats* stats) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo, "null argument");
        set_device(ctx);
        cudaStream_t s = ctx->stream;
        DevBuf d_dip((size_t)n_dipoles * 6 * 8, s), d_el((size_t)n_electrodes * 3 * 8, s),
            d_sq((size_t)n_squids * 6 * 8, s), d_ge((size_t)n_electrodes * n_dipoles * 8, s),
            d_gm((size_t)n_squids * n_dipoles * 8, s);
        if (n_dipoles) OMG_CUDA(cudaMemcpyAsync(d_dip.p, dipoles, n_dipoles * 48, cudaMemcpyHostToDevice, s));
        if (n_electrodes) OMG_CUDA(cudaMemcpyAsync(d_el.p, electrodes, n_electrodes * 24, cudaMemcpyHostToDevice, s));
        if (n_squids) OMG_CUDA(cudaMemcpyAsync(d_sq.p, squids, n_squids * 48, cudaMemcpyHostToDevice, s));
        int rc = omg_gain_dev(ctx, geo, precision, hm_integ, dsm_integ, d_dip.as<double>(), n_dipoles,
                              d_el.as<double>(), n_electrodes, d_sq.as<double>(), n_squids, d_ge.as<double>(),
                              d_gm.as<double>(), stats);
        if (rc != OMG_OK) throw Error(rc, g_last_error);
        if (n_electrodes && n_dipoles)
            OMG_CUDA(cudaMemcpyAsync(gain_eeg, d_ge.p, n_electrodes * n_dipoles * 8, cudaMemcpyDeviceToHost, s));
        if (n_squids && n_dipoles)
            OMG_CUDA(cudaMemcpyAsync(gain_meg, d_gm.p, n_squids * n_dipoles * 8, cudaMemcpyDeviceToHost, s));
        OMG_CUDA(cudaStreamSynchronize(s));
    });
}

}  // extern "C"
