// Internal declarations shared by the host library and the CUDA kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "openmeeg_gb300.h"

namespace omg {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define OMG_CUDA(x)                                                                                 \
    do {                                                                                            \
        cudaError_t e_ = (x);                                                                       \
        if (e_ != cudaSuccess)                                                                      \
            throw ::omg::Error(e_ == cudaErrorMemoryAllocation ? OMG_ERR_NOMEM : OMG_ERR_CUDA,      \
                               std::string(#x) + ": " + cudaGetErrorString(e_));                     \
    } while (0)

#define OMG_REQUIRE(cond, msg)                                                 \
    do {                                                                       \
        if (!(cond)) throw ::omg::Error(OMG_ERR_INVALID, (msg));               \
    } while (0)

constexpr double kK = 0.07957747154594767;          // 1/(4 pi), OpenMEEG/include/constants.h:23
constexpr double kMagFactor = 1e-7;                 // OpenMEEG/include/constants.h:22

// Per-triangle record sizes (doubles).
constexpr int SREC = 28;   // OperatorS data: p0 p1 p2 n area len[3] en[3] (25 used)
constexpr int PREC = 32;   // P1SingleLayerPotential data: p0 p1 p2 n area D[3] U[3] (31 used)
constexpr int QREC = 52;   // 16 quadrature points (48) + area (1), order-3 rule
constexpr int MAXQ = 16;
constexpr int kFarRecFloats = 96;   // floats per triangle of the mixed far-field records (GREC)

// --------------------------------------------------------------------------
// Host geometry: restates OpenMEEG's Geometry bookkeeping for meshes given as
// interfaces (OpenMEEG/src/geometry.cpp, interface.cpp, domain.h).
// --------------------------------------------------------------------------
// A domain boundary is an interface (a list of oriented meshes) and a side;
// `bounds` lists it mesh by mesh: the mesh, the side, the mesh's orientation
// in that interface (after the interface's global reorientation) and the
// index of the interface boundary within the domain (consecutive entries of
// one interface share it).
struct Boundary {
    int mesh;
    bool inside;
    int o = 1;
    int group = 0;
};
struct InterfaceBound {
    int iface;
    bool inside;
};
struct Domain {
    std::string name;
    std::vector<Boundary> bounds;
    double sigma;
    std::vector<InterfaceBound> ifb;
};
struct MeshPair {
    int m1, m2, orientation;
    double cS, cN, cD;
};

struct HostGeometry {
    int nmesh = 0;
    int64_t nv = 0, nt = 0;         // nv: vertices of all meshes, each mesh with its own copies
    int64_t nvg = 0;                // distinct vertices (the reference's unknowns); == nv when no mesh shares one
    std::vector<int64_t> vglob;     // mesh vertex copy -> distinct vertex (equal coordinates, geometry.h:100-108)
    bool shared = false;            // some meshes share vertices
    std::vector<std::vector<std::pair<int, int>>> ifaces;   // interfaces: (mesh, orientation +-1)
    std::vector<double> V;          // nv x 3
    std::vector<int32_t> T;         // nt x 3 global vertex ids
    std::vector<int64_t> vbeg, tbeg;
    std::vector<int> orient;        // interface orientation +-1
    std::vector<int> barrier, outermost;
    std::vector<Domain> domains;
    std::vector<MeshPair> pairs;
    std::vector<std::vector<int>> part_outermost;   // outermost meshes of each independent part
    std::vector<int> eeg_ifaces;                    // interfaces bounding sigma==0 domains, in visiting order
    // numbering (reference order): vertex copy v -> vglob[v]; triangle t -> tidx[t] (>= N for barrier meshes)
    std::vector<int64_t> tidx;
    int64_t N = 0, nP = 0;          // unknowns, triangle unknowns
    bool nested = true;
    // vertex -> incident triangles (CSR, triangle order)
    std::vector<int32_t> v2t_beg, v2t_tri;
    std::vector<int8_t> v2t_loc;    // local index of the vertex in that triangle

    int mesh_orientation(int d, int m) const;
    std::vector<int> domains_of(int m) const;
    double conductivity_jump(int m) const;
    void finalize();
    void recompute_coefficients();
};

HostGeometry build_geometry(int nmesh, const int64_t* nverts, const double* verts, const int64_t* ntris,
                            const int64_t* tris, int ndom, const int32_t* nb, const int32_t* bounds,
                            const double* sigma, const std::vector<std::string>& dom_names);
// Interfaces of several oriented meshes: interface i lists if_nm[i] signed
// 1-based mesh ids (+: normal orientation, -: opposite); domain boundaries are
// signed 1-based interface ids (-: inside).
HostGeometry build_geometry_interfaces(int nmesh, const int64_t* nverts, const double* verts, const int64_t* ntris,
                                       const int64_t* tris, int nif, const int32_t* if_nm, const int32_t* if_meshes,
                                       int ndom, const int32_t* nb, const int32_t* bounds, const double* sigma,
                                       const std::vector<std::string>& dom_names);
HostGeometry load_geometry_files(const std::string& geom, const std::string& cond);

// --------------------------------------------------------------------------
// Device geometry (flat arrays, internal numbering).
// Internal position of an unknown: triangle unknowns first, then identity
// padding up to a multiple of kPad, then vertices:
//   pos(triangle t) = tidx[t] - nv,  pos(vertex v) = nP + v,
// with nPt <= nP the true triangle-unknown count.  The padding keeps every
// block boundary of the factorization a multiple of 128 (aligned tensor-core
// tiles); padded rows/columns hold the identity and never touch the solution.
// --------------------------------------------------------------------------
constexpr int64_t kPad = 128;
struct DevGeom {
    int64_t nv = 0, nt = 0;
    int64_t nvg = 0;    // distinct vertices (reference numbering); == nv unless meshes share vertices
    int64_t N = 0;      // internal size nP + nv
    int64_t nP = 0;     // padded offset of the vertex unknowns
    int64_t nPt = 0;    // triangle unknowns
    int64_t Nref = 0;   // reference size nPt + nvg
    int nmesh = 0;
    double* V = nullptr;          // nv x 3
    int32_t* T = nullptr;         // nt x 3
    int32_t* tpos = nullptr;      // nt, internal position or -1
    double* srec = nullptr;       // nt x SREC
    double* prec = nullptr;       // nt x PREC
    double* qrec = nullptr;       // nt x QREC (order-3 points)
    int32_t* v2t_beg = nullptr;   // nv+1
    int32_t* v2t_tri = nullptr;
    int8_t* v2t_loc = nullptr;
    double* v2t_q = nullptr;      // per vertex-triangle slot: curl of the P1 basis over the area, 3 doubles
    int64_t* vglob = nullptr;     // copy -> distinct vertex; null when no mesh shares a vertex
};

// Device kernel launchers (assembly.cu / sources.cu / dense.cu).
struct Workspace;

void launch_prepare_triangles(const DevGeom& g, cudaStream_t s);
void launch_prepare_vertex_curls(const DevGeom& g, cudaStream_t s);
// S block: out(t1, t2) for t1 in [t1b,t1e), t2 in [t2b,t2e); `same` restricts to t2>=t1.
//   mode 0: write coeff*S into HM lower triangle at internal positions (ld)
//   mode 1: write S into tmp (n1 x n2 row-major, both halves when same)
void launch_S_block(const DevGeom& g, int64_t t1b, int64_t t1e, int64_t t2b, int64_t t2e, bool same, double coeff,
                    int order, double* hm, int64_t ld, double* tmp, int* err, cudaStream_t s);
void launch_D_block(const DevGeom& g, int64_t tab, int64_t tae, int64_t tbb, int64_t tbe, int order, double* tmp,
                    int* err, cudaStream_t s);
// rect: out(row = triangle unknown, col = vertex - vbb), column-major with ld, instead of the HM lower triangle
void launch_D_gather(const DevGeom& g, int64_t tab, int64_t tae, int64_t tbb, int64_t tbe, int64_t vbb, int64_t vbe,
                     double coeff, const double* tmp, double* hm, int64_t ld, cudaStream_t s, bool rect = false);
// s_contiguous_b: S(a, b) is contiguous along b (dense a-major temporaries; a block of the matrix whose mesh 2
// comes after mesh 1 in the internal order) rather than along a
void launch_N_block(const DevGeom& g, int64_t v1b, int64_t v1e, int64_t t1b, int64_t t1e, int64_t v2b, int64_t v2e,
                    int64_t t2b, int64_t t2e, bool same, double coeff, const double* hm_src, int64_t ld,
                    const double* tmp, double* hm, cudaStream_t s, bool rect, bool s_contiguous_b);
void launch_deflate(const DevGeom& g, const std::vector<std::pair<int64_t, int64_t>>& vranges, int64_t i_first,
                    int64_t nb, double* hm, int64_t ld, double* scratch, cudaStream_t s);
void launch_symmetrize_to_reference(const DevGeom& g, const double* hm_int, int64_t ld_int, double* out,
                                    int64_t ld_out, bool packed, cudaStream_t s);

int64_t kernel_launch_count();
void count_launch(int n = 1);

// Optional per-launch timing: when enabled, every launcher brackets its
// kernel with CUDA events on the launch stream; omg_profile_read() aggregates
// them per kernel name.
bool profiling_enabled();
void profile_record(const char* name, cudaEvent_t start, cudaEvent_t stop);
cudaEvent_t profile_event();
struct ProfScope {
    const char* name;
    cudaStream_t s;
    cudaEvent_t a = nullptr;
    ProfScope(const char* n, cudaStream_t st) : name(n), s(st) {
        if (profiling_enabled()) {
            a = profile_event();
            cudaEventRecord(a, s);
        }
    }
    ~ProfScope() {
        if (a) {
            cudaEvent_t b = profile_event();
            cudaEventRecord(b, s);
            profile_record(name, a, b);
        }
    }
};

// Grouped tensor-core products (tc_gemm.cu, gemm_tf32x3_grouped).  An operand
// map: K-major FP32 rows (`rows` rows of `kext` elements, row stride `ld`).
struct GemmOperand {
    const float* base;
    int64_t rows, kext, ld;
};
// One product C (M x N, column-major, ldc) = alpha A B^T with K-extent K:
// heads into C, remainders into Cr; A and B read through operand maps
// 4 set .. 4 set + 3 (Ah, Al, Bh, Bl) at rows ay_h / ay_l / by_h / by_l and
// K offsets ax / bx (multiples of 4).
struct GemmProduct {
    float* C;
    float* Cr;
    int64_t ldc, M, N, K;
    int set;
    int64_t ay_h, ay_l, by_h, by_l, ax, bx;
};

}  // namespace omg
