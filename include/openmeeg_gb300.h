/*
 * openmeeg_gb300.h -- C ABI of the GB300 symmetric-BEM forward path.
 *
 * Drop-in for OpenMEEG's forward path (HeadMat, DipSourceMat, Head2EEGMat,
 * Head2MEGMat, DipSource2MEGMat and the Gain* products).  Every entry point is
 * plain C: opaque handles, plain pointers, 64-bit sizes, an int status.
 *
 * Conventions
 *  - Return value: OMG_OK (0) or a negative OMG_ERR_* code; omg_last_error()
 *    gives a message for the calling thread.
 *  - Matrices are column-major float64, leading dimension = row count unless
 *    an `ld` argument says otherwise.
 *  - Unknowns follow the reference numbering (OpenMEEG/src/geometry.cpp:256-295):
 *    all vertices first, then the triangles of each mesh that is not a
 *    current barrier.
 *  - Functions named *_dev take device pointers (memory of the context's
 *    device); functions named *_host take host pointers and perform the
 *    host<->device copies themselves.
 *  - All work is queued on the context's stream; *_host functions and
 *    omg_context_synchronize() wait for it.
 */
#ifndef OPENMEEG_GB300_H
#define OPENMEEG_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OMG_OK                    0
#define OMG_ERR_INVALID          -1  /* bad argument or geometry (OMExceptions.H BadData/BadDomain...) */
#define OMG_ERR_CUDA             -2  /* CUDA runtime error */
#define OMG_ERR_NOT_DEFINITE     -3  /* HeadMat is not quasi-definite: factorization pivot of wrong sign */
#define OMG_ERR_NOT_CONVERGED    -4  /* iterative refinement did not reach its tolerance */
#define OMG_ERR_NOMEM            -5  /* device allocation failed */
#define OMG_ERR_IO               -6  /* file could not be read or parsed */
#define OMG_ERR_UNSUPPORTED      -7  /* valid request outside this build's scope */
#define OMG_ERR_TIMEOUT          -8  /* a bounded device-side wait gave up */
#define OMG_ERR_SINGULAR         -9  /* a dense LU met an exact zero pivot (LAPACK dgetrf info > 0) */

#define OMG_PREC_FP64             0  /* all-FP64 drop-in */
#define OMG_PREC_MIXED            1  /* FP32 far field + FP32 factorization + FP64-residual refinement */

typedef struct omg_context_s*  omg_context;
typedef struct omg_geometry_s* omg_geometry;
typedef struct omg_solver_s*   omg_solver;

/* Integrator(order, levels, tol) (OpenMEEG/include/integrator.h:192-196):
 * order 0..3 selects the 3/6/7/16-point Gauss rule, levels > 0 enables the
 * adaptive 4-way subdivision with relative tolerance tol. */
typedef struct {
    int32_t order;
    int32_t levels;
    double  tol;
} omg_integrator;

typedef struct {
    int64_t n_vertices;          /* all meshes */
    int64_t n_triangles;         /* all meshes */
    int64_t n_unknowns;          /* HeadMat dimension (nb_parameters - nb_current_barrier_triangles) */
    int64_t n_triangle_unknowns; /* unknowns carried by triangles */
    int32_t n_meshes;
    int32_t n_domains;
    int32_t n_mesh_pairs;        /* communicating mesh pairs (geometry.cpp:405-420) */
    int32_t nested;              /* 1 when every mesh bounds at most two domains */
} omg_geometry_info;

/* Per-call statistics of omg_gain_* (times in milliseconds, device clocks). */
typedef struct {
    double t_total_ms;
    double t_headmat_ms;
    double t_sources_ms;         /* DSM + H2EM + H2MM + DS2MM */
    double t_factor_ms;
    double t_solve_ms;           /* solves + refinement + gain GEMM */
    int32_t refinement_steps;    /* mixed precision only */
    int32_t residual_mode;       /* mixed: 1 tensor-core digits, 2 double-float on CUDA cores; FP64: 0 */
    double  final_residual;      /* max over RHS of ||b - HM x|| / ||b|| (mixed precision) */
    int64_t device_bytes;        /* peak device memory the call's own buffers held */
} omg_gain_stats;

/* ---- errors / context ---------------------------------------------------- */
const char* omg_last_error(void);
const char* omg_version(void);
int omg_context_create(int device, omg_context* out);
int omg_context_destroy(omg_context ctx);
/* Use an external CUDA stream (cudaStream_t passed as void*); NULL restores
 * the context's own stream. */
int omg_context_set_stream(omg_context ctx, void* stream);
int omg_context_synchronize(omg_context ctx);
/* Number of kernels this context has launched so far. */
int64_t omg_context_kernel_launches(omg_context ctx);

/* Per-kernel timing (process-wide): while enabled, every library kernel
 * launch is bracketed by CUDA events on its stream.  omg_profile_read waits
 * for the recorded events, writes per-kernel-name totals (names as 32-byte
 * NUL-padded strings, launch counts, milliseconds) for up to max_entries
 * kernels, stores the number written in *n_entries and clears the record. */
int omg_profile_enable(int32_t on);
int omg_profile_read(int32_t max_entries, char* names, int64_t* launches, double* total_ms, int32_t* n_entries);

/* ---- geometry ------------------------------------------------------------ *
 * Replaces Geometry(geom, cond) + Geometry::finalize
 * (OpenMEEG/include/geometry.h:67,211-249).  Meshes are given as interfaces
 * (.geom v1.1, one mesh per interface); `verts` concatenates the meshes'
 * vertices (n x 3, row-major), `tris` their triangles (local 0-based vertex
 * indices, m x 3).  Domain d has dom_nbounds[d] boundaries listed in
 * dom_bounds as signed 1-based mesh ids (-i: inside mesh i, +i: outside),
 * as in the .geom "Domain" lines (GeomFile.h:265-300). */
int omg_geometry_create(omg_context ctx, int32_t n_meshes, const int64_t* mesh_nverts, const double* verts,
                        const int64_t* mesh_ntris, const int64_t* tris, int32_t n_domains,
                        const int32_t* dom_nbounds, const int32_t* dom_bounds, const double* dom_sigma,
                        omg_geometry* out);
/* Geometry::load(geom, cond) for .geom v1.1 files whose interfaces are .tri
 * meshes (GeomFile.h:165-300, geometry.cpp:231-252, MeshIOs/tri.h). */
int omg_geometry_load(omg_context ctx, const char* geom_file, const char* cond_file, omg_geometry* out);
int omg_geometry_destroy(omg_geometry geo);
int omg_geometry_get_info(omg_geometry geo, omg_geometry_info* info);
/* Replace the domain conductivities (same domain order); coefficients and
 * barrier-dependent numbering must stay valid (no conductivity may change
 * to or from zero). */
int omg_geometry_set_conductivities(omg_geometry geo, const double* dom_sigma);

/* ---- assembly (device pointers) ------------------------------------------ */
/* HeadMat (OpenMEEG/src/assembleHeadMat.cpp:133-135): N x N symmetric, both
 * triangles written, column-major with leading dimension ld >= N. */
int omg_headmat_dev(omg_context ctx, omg_geometry geo, const omg_integrator* integ, int32_t precision,
                    double* hm, int64_t ld);
/* Same, in SymMatrix packed-upper storage (N(N+1)/2 doubles, i + j(j+1)/2). */
int omg_headmat_packed_dev(omg_context ctx, omg_geometry geo, const omg_integrator* integ, double* packed);
/* SourceMatrix<Dipole> (OpenMEEG/src/assembleSourceMat.cpp:66-104):
 * dipoles n x 6 row-major (x y z qx qy qz); out N x n.  domain = -1 looks up
 * each dipole's domain from its position; domain >= 0 forces that domain. */
int omg_dipsourcemat_dev(omg_context ctx, omg_geometry geo, const double* dipoles, int64_t n_dipoles,
                         const omg_integrator* integ, int32_t domain, double* dsm);
/* Head2EEGMat (OpenMEEG/src/assembleSensors.cpp:25-39): electrodes n x 3
 * row-major; out n x N dense (3 nonzeros per row), plus optionally the sparse
 * form: vertex unknown indices (n x 3) and weights (n x 3). */
int omg_head2eegmat_dev(omg_context ctx, omg_geometry geo, const double* electrodes, int64_t n_electrodes,
                        double* h2em, int64_t* sparse_cols, double* sparse_vals);
/* Head2MEGMat (OpenMEEG/src/assembleSensors.cpp:69-96) for point sensors:
 * squids n x 6 row-major (position, orientation); out n x N. */
int omg_head2megmat_dev(omg_context ctx, omg_geometry geo, const double* squids, int64_t n_squids, double* h2mm);
/* Head2MEGMat that allocates no device memory.  No counterpart in the
 * reference.  For callers that may not allocate once running (real-time
 * loops that cannot wait on the allocator, hosts that reserve the GPU's memory
 * up front, plugin hosts that forbid device allocations): the Ferguson pass
 * uses a fixed scratch array built into the library instead of a per-call
 * allocation.  Limit: n_squids x n_triangles <= OMG_NOALLOC_SCRATCH_DOUBLES.
 * The first call on a device sets up the scratch address (make it before any
 * stream capture); calls that overlap on the GPU share the array and race.
 * The call returns after its work on the context's stream has finished, as
 * omg_head2megmat_dev does.  Output and arguments as omg_head2megmat_dev. */
#define OMG_NOALLOC_SCRATCH_DOUBLES (4 * 1024 * 1024)
int omg_head2megmat_noalloc_dev(omg_context ctx, omg_geometry geo, const double* squids, int64_t n_squids,
                                double* h2mm);
/* DipSource2MEGMat (OpenMEEG/src/assembleSensors.cpp:133-159): out n_squids x n_dipoles. */
int omg_dipsource2megmat_dev(omg_context ctx, const double* dipoles, int64_t n_dipoles, const double* squids,
                             int64_t n_squids, double* ds2mm);

/* ---- adjoint (gradients) -------------------------------------------------- *
 * Building blocks of the vector-Jacobian products of the gain with respect to
 * the conductivities and the dipoles (no counterpart in the reference, which
 * has no derivatives). */
typedef struct {
    int64_t vbeg, vend;        /* vertex unknowns of the mesh (reference numbering) */
    int64_t tri_unknown;       /* first triangle unknown, -1 for a current barrier */
    int64_t n_triangles;
    int32_t barrier;           /* touches a zero-conductivity domain */
    int32_t orientation;       /* interface orientation (+1/-1) */
    int32_t outermost;
    int32_t reserved;
} omg_mesh_layout;
typedef struct {
    int32_t m1, m2, orientation, reserved;
    double cS, cN, cD;         /* S, N, D block coefficients (assembleHeadMat.cpp:92-95) */
} omg_mesh_pair;
int omg_geometry_get_layout(omg_geometry geo, int32_t max_meshes, omg_mesh_layout* out);
int omg_geometry_get_pairs(omg_geometry geo, int32_t max_pairs, omg_mesh_pair* out, int32_t* n_pairs);
/* Domain index of each dipole position (Geometry::domain(point)); -1 if none. */
int omg_dipole_domains_dev(omg_context ctx, omg_geometry geo, const double* dipoles, int64_t n_dipoles,
                           int32_t* domains);
/* Head2MEGMat contribution of one mesh with a unit conductivity jump
 * (assembleFerguson.cpp:18-31 without the jump factor): out n_squids x N. */
int omg_head2megmat_mesh_dev(omg_context ctx, omg_geometry geo, const double* squids, int64_t n_squids,
                             int32_t mesh, double* out);
/* d/d(position, moment) of sum_rows U[row, j] DSM[row, j] for every dipole j:
 * U is N x n_dipoles (reference numbering, leading dimension ldu); out is
 * n_dipoles x 6 row-major (dx dy dz dqx dqy dqz).  Same integrator and
 * adaptive trees as omg_dipsourcemat_dev. */
int omg_dipsourcemat_vjp_dev(omg_context ctx, omg_geometry geo, const double* dipoles, int64_t n_dipoles,
                             const omg_integrator* integ, int32_t domain, const double* U, int64_t ldu,
                             double* out);
/* C = alpha op(A) op(B) + beta C in FP64 (column-major; trans = 1 transposes). */
int omg_gemm_f64_dev(omg_context ctx, int32_t trans_a, int32_t trans_b, int64_t m, int64_t n, int64_t k, double alpha,
                     const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc);

/* ---- dense solve ---------------------------------------------------------- *
 * Replaces SymMatrix::solveLin / linsolve (OpenMEEGMaths/src/symmatrix.cpp:133-152,
 * OpenMEEG/include/gain.h:52-57): the solver owns a factorization of HeadMat.
 * FP64: quasi-definite L D L^T with D = diag(+1 on triangle unknowns, -1 on
 * vertex unknowns).  Mixed: the same factorization in FP32 plus FP64-residual
 * iterative refinement against the FP64 HeadMat. */
int omg_solver_create(omg_context ctx, omg_geometry geo, const omg_integrator* integ, int32_t precision,
                      omg_solver* out);
/* Factor a caller-provided HeadMat (dense, column-major, reference
 * numbering, lower triangle read) -- SymMatrix::solveLin on an existing HM. */
int omg_solver_from_headmat_dev(omg_context ctx, omg_geometry geo, const double* hm, int64_t ld,
                                int32_t precision, omg_solver* out);
/* In place: B (N x nrhs, leading dimension ldb) <- HeadMat^-1 B.  Mixed
 * precision: if the refinement stalls above its tolerance, the head matrix is
 * rebuilt and solved in FP64 (quasi-definite LDL^T, or the pivoted LU), and the
 * solver stays FP64 from then on. */
int omg_solver_solve_dev(omg_solver s, double* b, int64_t ldb, int64_t nrhs);
/* Mixed-precision refinement controls: stop when the predicted relative error
 * of the solution is below tol (default 1e-6), after at most max_steps
 * residual steps (default 10). */
int omg_solver_set_refinement(omg_solver s, double tol, int32_t max_steps);
int omg_solver_destroy(omg_solver s);

/* ---- gain ------------------------------------------------------------------ *
 * GainEEGadjoint / GainMEGadjoint / GainEEGMEGadjoint (OpenMEEG/include/gain.h:78-136):
 * assemble HeadMat, factor it, solve for the sensor rows, contract with the
 * DipSourceMat and add DipSource2MEGMat.  Any of electrodes/squids may be
 * NULL (count 0).  gain_eeg: n_electrodes x n_dipoles; gain_meg: n_squids x
 * n_dipoles.  `hm_integ` / `dsm_integ` may be NULL for the reference
 * defaults (3,0,0.005) and (3,10,0.001). */
int omg_gain_dev(omg_context ctx, omg_geometry geo, int32_t precision, const omg_integrator* hm_integ,
                 const omg_integrator* dsm_integ, const double* dipoles, int64_t n_dipoles,
                 const double* electrodes, int64_t n_electrodes, const double* squids, int64_t n_squids,
                 double* gain_eeg, double* gain_meg, omg_gain_stats* stats);
/* Same with host buffers (inputs copied in, gains copied out). */
int omg_gain_host(omg_context ctx, omg_geometry geo, int32_t precision, const omg_integrator* hm_integ,
                  const omg_integrator* dsm_integ, const double* dipoles, int64_t n_dipoles,
                  const double* electrodes, int64_t n_electrodes, const double* squids, int64_t n_squids,
                  double* gain_eeg, double* gain_meg, omg_gain_stats* stats);

/* ---- gains from an explicit inverse ----------------------------------------
 * GainEEG (OpenMEEG/include/gain.h:69-76; om_gain -EEG, apps/gain.cpp:65-80):
 * gain = (H2EM HMinv) DSM for the inverse head matrix HMinv that om_minverser
 * writes (SymMatrix::invert, OpenMEEGMaths/include/symmatrix.h:280-300).
 * hminv: N x N column-major with leading dimension ld (packed = 0), or
 * SymMatrix packed-upper storage, entry (i, j), i <= j, at i + j(j+1)/2
 * (packed = 1, ld ignored).  H2EM is the sparse matrix of the reference's
 * SparseMatrix in coordinate form: nnz (row, column, value) triplets with rows
 * in [0, n_electrodes) and columns in [0, N) (device arrays; duplicates add).
 * dsm: N x n_dipoles (leading dimension N); gain: n_electrodes x n_dipoles.
 * precision OMG_PREC_FP64: FP64 CUDA-core products; OMG_PREC_MIXED: the
 * FP64-accurate fixed-point digit GEMM on the tensor cores. */
int omg_gain_eeg_dev(omg_context ctx, int64_t N, const double* hminv, int64_t ld, int32_t packed,
                     const double* dsm, int64_t n_dipoles, int64_t n_electrodes, int64_t nnz,
                     const int64_t* h2em_rows, const int64_t* h2em_cols, const double* h2em_vals, int32_t precision,
                     double* gain);
/* GainMEG (OpenMEEG/include/gain.h:60-67; om_gain -MEG, apps/gain.cpp:105-122):
 * gain = DS2MM + (H2MM HMinv) DSM.  h2mm: n_squids x N, ds2mm: n_squids x
 * n_dipoles (leading dimensions = row counts); other arguments as
 * omg_gain_eeg_dev. */
int omg_gain_meg_dev(omg_context ctx, int64_t N, const double* hminv, int64_t ld, int32_t packed,
                     const double* dsm, int64_t n_dipoles, const double* h2mm, int64_t n_squids, const double* ds2mm,
                     int32_t precision, double* gain);

/* ---- cortical mapping -------------------------------------------------------
 * CorticalMat (OpenMEEG/src/assembleHeadMat.cpp:168-236; om_assemble -CM with
 * zero or two numbers): out = P pinv(P^T A P) P^T M^T, N x n_electrodes
 * column-major (N: the reference's unknowns), mapping electrode potentials to
 * the unknowns.  M is Head2EEGMat (n_electrodes x N) as device triplets, as for
 * omg_gain_eeg_dev; P projects on the null space of the head-matrix rows
 * outside the cortex (the head matrix assembled without the cortex mesh's own
 * block, assembleHeadMat.cpp:137-166); A = M^T M + alpha RR_vertices +
 * beta RR_triangles with RR the gradient norms of every mesh
 * (Mesh::gradient_norm2, mesh.cpp:160-205); alpha < 0 selects
 * alpha = ||M^T M||_F / (1000 ||RR_vertices||_F) and beta = 50000 alpha.  The
 * cortex is the one mesh of the one interface bounding `domain` (an index into
 * the geometry's domains), else OMG_ERR_INVALID.  Computed as the KKT system
 * [A mat^T; mat 0] [X; L] = [M^T; 0] by an FP64 LU with partial pivoting: the
 * same X whenever P^T A P has the rank of P.  projector_in (optional, N x N,
 * device): a projector from the reference's cache file, used instead of the
 * head matrix (X = P (P A P + I - P)^-1 P M^T); projector_out (optional, N x N):
 * receives P = I - mat^T (mat mat^T)^-1 mat, the matrix the reference caches. */
int omg_corticalmat_dev(omg_context ctx, omg_geometry geo, const omg_integrator* integ, int32_t domain,
                        int64_t n_electrodes, int64_t nnz, const int64_t* h2em_rows, const int64_t* h2em_cols,
                        const double* h2em_vals, double alpha, double beta, const double* projector_in,
                        double* projector_out, double* out);
/* CorticalMat2 (assembleHeadMat.cpp:238-323; om_assemble -CM with one number):
 * out = (G^-1 H^T (H G^-1 H^T)^-1) restricted to the electrode columns,
 * N x n_electrodes, with H = [the head-matrix rows outside the cortex; M] and G
 * the gradient norms whose triangle-triangle entries the reference scales by
 * gamma once per ordered pair (gamma^2 off the diagonal).  Solved as
 * [G H^T; H 0] [X; L] = [0; E].  rows_in (optional, device, n_rows x N
 * column-major): the head-matrix rows from the reference's cache file instead
 * of assembling them; rows_out (optional, n_rows x N): receives them.  An
 * exactly singular system returns OMG_ERR_SINGULAR. */
int omg_corticalmat2_dev(omg_context ctx, omg_geometry geo, const omg_integrator* integ, int32_t domain,
                         int64_t n_electrodes, int64_t nnz, const int64_t* h2em_rows, const int64_t* h2em_cols,
                         const double* h2em_vals, double gamma, const double* rows_in, double* rows_out,
                         double* out);
/* n_rows: the head-matrix rows outside the cortex of `domain` (N minus the
 * cortex's vertices and triangles). */
int omg_cortical_rows(omg_geometry geo, int32_t domain, int64_t* n_rows);

/* ---- surface sources -------------------------------------------------------
 * SurfSourceMat (OpenMEEG/src/assembleSourceMat.cpp:22-64, assembleSourceMat.h:20):
 * a triangulated source surface (host arrays: vertices n x 3 row-major,
 * triangles m x 3 0-based) inside one conducting domain of the geometry; out
 * is N x n_verts column-major in the reference numbering.  The default
 * integrator is the reference's (3, 0, 0.005); adaptive integration is not
 * supported.  A source mesh whose vertices lie in different domains is
 * rejected (the reference's OverlappingSourceMesh). */
int omg_surfsourcemat_dev(omg_context ctx, omg_geometry geo, const double* verts, int64_t n_verts,
                          const int64_t* tris, int64_t n_tris, const omg_integrator* integ, double* ssm);
/* SurfSource2MEGMat (OpenMEEG/src/assembleSensors.cpp:102-125): squids on the
 * device (n x 6), source mesh from host arrays; out n_squids x n_verts,
 * column-major. */
int omg_surfsource2megmat_dev(omg_context ctx, const double* verts, int64_t n_verts, const int64_t* tris,
                              int64_t n_tris, const double* squids, int64_t n_squids, double* ss2mm);

/* ---- internal potentials ----------------------------------------------------
 * Points (device, n x 3) are located in the geometry's domains; those in a
 * zero-conductivity domain are dropped, as the reference does, and the rest
 * keep their input order.  *n_kept returns their count; out must hold
 * n_points x columns doubles and receives an n_kept x columns column-major
 * matrix (leading dimension n_kept).  A point in no domain is an error.
 *
 * Surf2VolMat (OpenMEEG/src/assembleHeadMat.cpp:325-363, assemble.h:33;
 * PartialBlock, OpenMEEG/include/operators.h:302-331): columns are the Nref
 * surface unknowns in the reference numbering. */
int omg_surf2volmat_dev(omg_context ctx, omg_geometry geo, const double* points, int64_t n_points, double* out,
                        int64_t* n_kept);
/* DipSource2InternalPotMat (OpenMEEG/src/assembleSourceMat.cpp:154-187,
 * assembleSourceMat.h:32): columns are the dipoles (device, n x 6); domain -1
 * takes each dipole's own domain, domain >= 0 forces that domain index (the
 * reference's domain_name argument). */
int omg_dipsource2internalpotmat_dev(omg_context ctx, omg_geometry geo, const double* dipoles, int64_t n_dipoles,
                                     const double* points, int64_t n_points, int32_t domain, double* out,
                                     int64_t* n_kept);

/* EITSourceMat (OpenMEEG/src/assembleSourceMat.cpp:109-152, assembleSourceMat.h:31):
 * electrode positions (device, n x 3) and radii (device, n; NULL for point
 * electrodes); the injection triangles and weights follow
 * Sensors::findInjectionTriangles (OpenMEEG/src/sensors.cpp:167-215).  out is
 * Nref x n_electrodes, column-major.  Default integrator (3, 0, 0.005). */
int omg_eitsourcemat_dev(omg_context ctx, omg_geometry geo, const double* positions, const double* radii,
                         int64_t n_electrodes, const omg_integrator* integ, double* out);

/* ---- batched forward (no reference counterpart) -----------------------------
 * Many head models, each with its own geometry, dipoles and sensors, computed
 * by one captured CUDA graph: every model's forward is the adjoint gain of
 * omg_gain_dev (GainEEGadjoint / GainMEGadjoint, OpenMEEG/include/gain.h:78-136)
 * in the given precision with the default integrators, and the models run as
 * parallel branches (one stream each).  omg_batch_create makes one uncaptured
 * planning run (which fixes the mixed assembly's near-pair lists, the number of
 * refinement steps and the DipSourceMat row ranges), picks the number of
 * branches (n_branches = 0: timed over 1, 2, 4, 8, 16 within 70% of free
 * device memory, cached by batch signature in the file named by the
 * OMG_TUNE_CACHE environment variable) and captures the graph;
 * omg_batch_run replays it on the context's stream and waits for it.
 * Geometries stay referenced by the batch and must not be used by other calls
 * while a batch call runs.  Changing a geometry's conductivities makes the
 * next run plan and capture again.  New dipoles (omg_batch_set_dipoles, same
 * count) must lie in domains whose rows the plan covers, else the run fails
 * with OMG_ERR_INVALID. */
typedef struct omg_batch_s* omg_batch;
typedef struct {
    omg_geometry geometry;
    const double* dipoles;    int64_t n_dipoles;      /* host, n x 6 row-major */
    const double* electrodes; int64_t n_electrodes;   /* host, n x 3 row-major */
    const double* squids;     int64_t n_squids;       /* host, n x 6 row-major */
} omg_batch_model;
typedef struct {
    int32_t n_models;
    int32_t n_branches;
    int32_t precision;
    int32_t max_refine_steps;
    int64_t launches_per_run;       /* kernel launches recorded in the graph */
    int64_t graph_nodes;
    int64_t graph_bytes_estimate;   /* device memory of the branches' largest models */
    double tuned_ms;                /* replay time of the chosen branch count (0: not timed) */
} omg_batch_info;
int omg_batch_create(omg_context ctx, int32_t n_models, const omg_batch_model* models, int32_t precision,
                     int32_t n_branches, omg_batch* out);
int omg_batch_run(omg_batch batch);
/* Device pointers owned by the batch: EEG gain n_electrodes x n_dipoles and
 * MEG gain n_squids x n_dipoles, column-major; valid until destroy. */
int omg_batch_gain_dev(omg_batch batch, int32_t model, const double** gain_eeg, const double** gain_meg);
int omg_batch_set_dipoles(omg_batch batch, int32_t model, const double* dipoles);
int omg_batch_get_info(omg_batch batch, omg_batch_info* info);
int omg_batch_destroy(omg_batch batch);

#ifdef __cplusplus
}
#endif

#endif /* OPENMEEG_GB300_H */
