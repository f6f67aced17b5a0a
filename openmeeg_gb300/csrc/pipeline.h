// Internal stages of the forward pipeline shared by the single-model entry
// points (api.cpp) and the batched, graph-captured forward (batch.cpp).
// Every stage enqueues on the stream of the context its handle points to.
#pragma once

#include <string>
#include <utility>
#include <vector>

#include <functional>

#include "handles.h"

struct omg_solver_s {
    omg_context ctx = nullptr;
    omg_geometry geo = nullptr;
    int precision = OMG_PREC_FP64;
    int64_t N = 0, nP = 0;
    std::vector<int64_t> bounds;            // block boundaries (include nP)
    DevBuf A64;                             // FP64: factor (lower).  Mixed: the head matrix as float pairs
                                            // (hi, lo; 2 x N x N floats) for the refinement residual
    DevBuf A32;                             // mixed: FP32 factor (TF32 heads after the split), ld = ld32
    DevBuf A32r;                            // mixed: FP32 remainders of the factor
    DevBuf W;                               // mixed: K-major head/remainder copies of every panel
    DevBuf Linv32;                          // mixed: inverses of the 128 x 128 diagonal blocks
    std::vector<int64_t> w_off;             // offset (floats) of panel b's heads; remainders follow
    int64_t ld32 = 0;
    // mixed: refinement residual on the tensor cores from fixed-point digits of
    // the FP64 head matrix (nda planes of base-2^beta digits, row exponents);
    // false: double-float residual on the CUDA cores from A64
    bool tc_residual = true;
    int residual_choice = -1;               // -1: decide at factorization (memory, OMG_RESIDUAL); 0/1: given
    DevBuf Adig, rexp;
    // 6 digits of 7 bits per operand, digit pairs up to level 7 (21 pairs): residual entries within ~2^-42 of
    // n max|A_i.| max|X_.c| -- below what a plain FP64 product accumulates over n ~ 1e4-1e5 terms, and far below
    // what one refinement step needs (its correction is ~1e-4 of x)
    int nda = 6, ndx = 6, beta = 7, lmax = 7;
    bool persistent = false;                // outlives the call that made it (public solver handle)
    double refine_tol = 1e-6;               // stop when corrections are this small relative to x
    int max_refine = 10;
    int last_steps = 0;
    double last_residual = 0.0;
    double last_correction = 0.0;
    int sweep_ctas = 0;                     // mixed: CTAs of a persistent sweep (0: one per SM)
    // pivoted fallback: the quasi-definite LDL^T met a pivot of the wrong sign, so A64 holds the FP64 LU
    // factors with partial pivoting of the whole matrix (any nonsingular matrix, as the reference's
    // Bunch-Kaufman DSPTRF) and perm its row order
    bool lu = false;
    DevBuf perm;
    // the head matrix again (assembled or copied in), for the FP64 solve a stalled refinement falls back to
    std::function<DevBuf()> rebuild;
};

// Near-pair lists of a geometry's mixed-precision assembly, one per mesh pair.
// They depend on the meshes only, so a recorded plan lets the assembly run
// without reading the pair counts back to the host (a requirement of stream
// capture).
struct NearPlan {
    bool recorded = false;
    std::vector<int> count;
    std::vector<DevBuf> list;    // persistent, max(count, 1) int2 each
    DevBuf counter;              // persistent, one int per mesh pair
};

template <typename F>
inline int guarded(F&& f) {
    try {
        f();
        return OMG_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return OMG_ERR_NOMEM;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return OMG_ERR_INVALID;
    }
}

void set_device(omg_context ctx);
void ensure_aux(omg_context ctx);
void release_context(omg_context ctx);
void release_geometry(omg_geometry geo);
void reset_err(omg_context ctx);
void check_err(omg_context ctx, const char* what);
omg_integrator default_hm_integrator();
omg_integrator default_dsm_integrator();
void check_integrator(const omg_integrator& it, bool allow_adaptive);
void ensure_order(omg_geometry g, int order);
void ensure_gg_tables(omg_geometry g);
// skip_self_mesh >= 0: that mesh's own block is left out (HeadMatrix with AllButBlock, assembleHeadMat.cpp:65-69)
void assemble_headmat_internal(omg_geometry g, const omg_integrator& integ, double* hm, int64_t ld,
                               int skip_self_mesh = -1);
void assemble_headmat_mixed(omg_geometry g, const omg_integrator& integ, double* hm, int64_t ld,
                            NearPlan* plan = nullptr);
void solver_factor(omg_solver sv, DevBuf&& hm, bool check = true);
// solver_factor; on OMG_ERR_NOT_DEFINITE the matrix `again()` returns (the same head matrix, rebuilt) is
// factored by the pivoted FP64 LU instead
void solver_factor_or_pivot(omg_solver sv, DevBuf&& hm, const std::function<DevBuf()>& again);
void solver_solve_internal(omg_solver sv, double* B, int64_t ldb, int64_t nrhs);
void solve_mixed_fixed(omg_solver sv, double* B, int64_t ldb, int64_t nrhs, int residual_steps, double* d_est);
void dsm_internal(omg_geometry g, const double* dip, int64_t nd, const omg_integrator& integ, int domain, int perm,
                  double* out, int64_t ldo, int precision = OMG_PREC_FP64, std::vector<int>* meshes_used = nullptr,
                  uint64_t allowed_domains = 0, DevBuf* dom_out = nullptr);
// Row ranges (internal numbering, merged) where the DipSourceMat of dipoles in
// the given source meshes' domains can be nonzero.
std::vector<std::pair<int64_t, int64_t>> gain_row_ranges(omg_geometry geo, const std::vector<int>& src_meshes);
// G = Y^T DSM restricted to `rows`: EEG rows of Y first (ne), then MEG (nm,
// accumulated onto gmeg, which already holds DipSource2MEGMat).  FP64: CUDA-core
// FP64 GEMM; mixed: FP64-accurate digit GEMM on the tensor cores.
void gain_contract(const std::vector<std::pair<int64_t, int64_t>>& rows, const double* Y, int64_t N, int64_t ne,
                   int64_t nm, const double* DSM, int64_t nd, double* geeg, double* gmeg, cudaStream_t s,
                   int precision, int* err);
