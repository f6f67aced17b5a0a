// BEM assembly kernels for sm_103a: HeadMat blocks (S, D, N, deflation),
// DipSourceMat, the sensor matrices and the triangle preprocessing they share.
//
// Layout in HBM.  The head matrix lives as a dense N x N column-major FP64
// array in the solver's internal numbering -- triangle unknowns first, then
// vertex unknowns (the reference's [V | P] order rotated by n_vertices) --
// and only its lower triangle is written.  Per-triangle records (OperatorS
// data, P1 single-layer data, quadrature points) are precomputed once and
// staged tile by tile into shared memory with bulk (TMA) copies.
//
// Each kernel restates the reference loop it replaces; the per-pair work is
// the reference's analytic inner integral times its Gauss outer rule, so the
// FP64 results agree with the reference to rounding.
#include <algorithm>
#include <cstdio>
#include <string>
#include <tuple>
#include <vector>

#include "device_common.cuh"
#include "handles.h"
#include "omg_internal.h"

namespace omg {

using dev::d3;

// Gauss rules of 3/6/7/16 points (OpenMEEG/include/integrator.h:260-318;
// Bonnet's tables).  The digits are those of the reference: parity at 1e-10
// requires the same truncated nodes.  [order][point] = {b0, b1, b2, weight}.
__constant__ double c_rules[4][16][4] = {
    {{0.166666666666667, 0.166666666666667, 0.666666666666667, 0.333333333333334},
     {0.166666666666667, 0.666666666666667, 0.166666666666667, 0.333333333333334},
     {0.666666666666667, 0.166666666666667, 0.166666666666667, 0.333333333333334}},
    {{0.445948490915965, 0.445948490915965, 0.108103018168070, 0.223381589678010},
     {0.445948490915965, 0.108103018168070, 0.445948490915965, 0.223381589678010},
     {0.108103018168070, 0.445948490915965, 0.445948490915965, 0.223381589678010},
     {0.091576213509771, 0.091576213509771, 0.816847572980458, 0.109951743655322},
     {0.091576213509771, 0.816847572980458, 0.091576213509771, 0.109951743655322},
     {0.816847572980458, 0.091576213509771, 0.091576213509771, 0.109951743655322}},
    {{0.333333333333333, 0.333333333333333, 0.333333333333333, 0.2250},
     {0.470142064105115, 0.470142064105115, 0.059715871789770, 0.132394152788506},
     {0.470142064105115, 0.059715871789770, 0.470142064105115, 0.132394152788506},
     {0.059715871789770, 0.470142064105115, 0.470142064105115, 0.132394152788506},
     {0.101286507323456, 0.101286507323456, 0.797426985353088, 0.125939180544828},
     {0.101286507323456, 0.797426985353088, 0.101286507323456, 0.125939180544828},
     {0.797426985353088, 0.101286507323456, 0.101286507323456, 0.125939180544828}},
    {{0.333333333333333, 0.333333333333333, 0.333333333333333, 0.144315607677786},
     {0.081414823414554, 0.459292588292722, 0.459292588292722, 0.095091634267284},
     {0.459292588292722, 0.081414823414554, 0.459292588292722, 0.095091634267284},
     {0.459292588292722, 0.459292588292722, 0.081414823414554, 0.095091634267284},
     {0.898905543365937, 0.050547228317031, 0.050547228317031, 0.032458497623198},
     {0.050547228317031, 0.898905543365937, 0.050547228317031, 0.032458497623198},
     {0.050547228317031, 0.050547228317031, 0.898905543365937, 0.032458497623198},
     {0.658861384496479, 0.170569307751760, 0.170569307751761, 0.103217370534718},
     {0.170569307751760, 0.658861384496479, 0.170569307751761, 0.103217370534718},
     {0.170569307751760, 0.170569307751761, 0.658861384496479, 0.103217370534718},
     {0.008394777409957, 0.728492392955404, 0.263112829634639, 0.027230314174434},
     {0.728492392955404, 0.008394777409957, 0.263112829634639, 0.027230314174434},
     {0.728492392955404, 0.263112829634639, 0.008394777409957, 0.027230314174434},
     {0.008394777409957, 0.263112829634639, 0.728492392955404, 0.027230314174434},
     {0.263112829634639, 0.008394777409957, 0.728492392955404, 0.027230314174434},
     {0.263112829634639, 0.728492392955404, 0.008394777409957, 0.027230314174434}}};
__constant__ int c_nbpts[4] = {3, 6, 7, 16};

static int64_t g_launches = 0;
int64_t kernel_launch_count() { return g_launches; }
void count_launch(int n) { g_launches += n; }

// ---- launch profiler (events pooled; aggregated on read) ----
struct ProfEntry {
    const char* name;
    cudaEvent_t a, b;
};
static bool g_prof = false;
static std::vector<ProfEntry> g_prof_entries;
static std::vector<cudaEvent_t> g_prof_pool;
bool profiling_enabled() { return g_prof; }
cudaEvent_t profile_event() {
    if (!g_prof_pool.empty()) {
        cudaEvent_t e = g_prof_pool.back();
        g_prof_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}
void profile_record(const char* name, cudaEvent_t a, cudaEvent_t b) { g_prof_entries.push_back({name, a, b}); }
void profile_enable(bool on) { g_prof = on; }
// Aggregates recorded launches per name (synchronizes on each event).
std::vector<std::tuple<std::string, int64_t, double>> profile_collect() {
    std::vector<std::tuple<std::string, int64_t, double>> out;
    for (auto& e : g_prof_entries) {
        cudaEventSynchronize(e.b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e.a, e.b);
        bool found = false;
        for (auto& o : out)
            if (std::get<0>(o) == e.name) {
                std::get<1>(o) += 1;
                std::get<2>(o) += ms;
                found = true;
            }
        if (!found) out.emplace_back(e.name, 1, (double)ms);
        g_prof_pool.push_back(e.a);
        g_prof_pool.push_back(e.b);
    }
    g_prof_entries.clear();
    return out;
}

static inline void check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error(OMG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    count_launch();
}

static inline unsigned nblocks(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// Quadrature point: sum_j b_j p_j accumulated from zero without contraction,
// as Vect3::multadd does (integrator.h:214-225).
__device__ __forceinline__ d3 bary_point(const double* r, d3 p0, d3 p1, d3 p2) {
    d3 v;
    v.x = __dadd_rn(__dadd_rn(__dmul_rn(r[0], p0.x), __dmul_rn(r[1], p1.x)), __dmul_rn(r[2], p2.x));
    v.y = __dadd_rn(__dadd_rn(__dmul_rn(r[0], p0.y), __dmul_rn(r[1], p1.y)), __dmul_rn(r[2], p2.y));
    v.z = __dadd_rn(__dadd_rn(__dmul_rn(r[0], p0.z), __dmul_rn(r[1], p1.z)), __dmul_rn(r[2], p2.z));
    return v;
}

// ---------------------------------------------------------------------------
// Triangle preprocessing: normal/area (triangle.h:57-62), OperatorS edge data
// (analytics.h:22-30), P1SingleLayerPotential edge data (analytics.h:81-85),
// and the points of the `order` rule.
// ---------------------------------------------------------------------------
__global__ void prepare_triangles_kernel(int64_t nt, const double* __restrict__ V, const int32_t* __restrict__ T,
                                         int order, double* srec, double* prec, double* qrec) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const d3 p0 = dev::ld3(V + 3 * (int64_t)T[3 * t]);
    const d3 p1 = dev::ld3(V + 3 * (int64_t)T[3 * t + 1]);
    const d3 p2 = dev::ld3(V + 3 * (int64_t)T[3 * t + 2]);
    d3 nn = dev::cross(p1 - p0, p2 - p0);
    const double nrm = dev::norm(nn);
    const double area = 0.5 * nrm;
    const d3 n = nn * (1.0 / nrm);
    double* s = srec + t * SREC;
    const d3 P[3] = {p0, p1, p2};
    for (int i = 0; i < 3; ++i) {
        s[3 * i] = P[i].x;
        s[3 * i + 1] = P[i].y;
        s[3 * i + 2] = P[i].z;
    }
    s[9] = n.x; s[10] = n.y; s[11] = n.z;
    s[12] = area;
    for (int i = 0; i < 3; ++i) {
        const d3 vref = P[i] - P[(i + 1) % 3];
        const double len = dev::norm(vref);
        const d3 unit = dev::mk(vref.x / len, vref.y / len, vref.z / len);
        const d3 en = dev::cross(n, unit);
        s[13 + i] = len;
        s[16 + 3 * i] = en.x; s[17 + 3 * i] = en.y; s[18 + 3 * i] = en.z;
    }
    for (int i = 25; i < SREC; ++i) s[i] = 0.0;
    double* p = prec + t * PREC;
    for (int i = 0; i < 13; ++i) p[i] = s[i];
    const d3 D[3] = {p1 - p0, p2 - p1, p0 - p2};
    for (int i = 0; i < 3; ++i) {
        const double dn = dev::norm(D[i]);
        p[13 + 3 * i] = D[i].x; p[14 + 3 * i] = D[i].y; p[15 + 3 * i] = D[i].z;
        p[22 + 3 * i] = D[i].x / dn; p[23 + 3 * i] = D[i].y / dn; p[24 + 3 * i] = D[i].z / dn;
    }
    p[31] = 0.0;
    double* q = qrec + t * QREC;
    const int np = c_nbpts[order];
    for (int k = 0; k < MAXQ; ++k) {
        d3 v = dev::mk(0, 0, 0);
        if (k < np) v = bary_point(c_rules[order][k], p0, p1, p2);
        q[3 * k] = v.x; q[3 * k + 1] = v.y; q[3 * k + 2] = v.z;
    }
    q[48] = area;
    for (int i = 49; i < QREC; ++i) q[i] = 0.0;
}

void launch_prepare_triangles_order(const DevGeom& g, int order, cudaStream_t s) {
    ProfScope prof_("prepare_triangles", s);
    prepare_triangles_kernel<<<nblocks(g.nt, 128), 128, 0, s>>>(g.nt, g.V, g.T, order, g.srec, g.prec, g.qrec);
    check_launch("prepare_triangles");
}
void launch_prepare_triangles(const DevGeom& g, cudaStream_t s) { launch_prepare_triangles_order(g, 3, s); }

// Lower-triangle address of (a, b) in the internal column-major matrix.
__device__ __forceinline__ int64_t lower_at(int64_t a, int64_t b, int64_t ld) {
    return a >= b ? a + b * ld : b + a * ld;
}

// ---------------------------------------------------------------------------
// S block (DiagonalBlock::S operators.h:209-237, NonDiagonalBlock::S :391-425):
// S(t1,t2) = coeff * integral over t2 (Gauss rule) of OperatorS(t1).
// One CTA per TI x TJ tile; t1 OperatorS records and t2 quadrature records
// are bulk-copied into shared memory.  One thread per (t1,t2) pair.
// ---------------------------------------------------------------------------
constexpr int S_TI = 16, S_TJ = 64, S_THREADS = 256;

__global__ void __launch_bounds__(S_THREADS) s_block_kernel(const double* __restrict__ srec,
                                                            const double* __restrict__ qrec, int64_t t1b, int64_t n1,
                                                            int64_t t2b, int64_t n2, int same, double coeff,
                                                            int order, const int32_t* __restrict__ tpos, double* hm,
                                                            int64_t ld, double* tmp, int* err) {
    extern __shared__ __align__(16) double smem[];
    __shared__ __align__(8) uint64_t bar;
    const int64_t i0 = (int64_t)blockIdx.y * S_TI, j0 = (int64_t)blockIdx.x * S_TJ;
    if (same && j0 + S_TJ <= i0) return;   // tile strictly below the diagonal
    const int ni = (int)(n1 - i0 < (int64_t)S_TI ? n1 - i0 : (int64_t)S_TI), nj = (int)(n2 - j0 < (int64_t)S_TJ ? n2 - j0 : (int64_t)S_TJ);
    double* sS = smem;                 // ni x SREC
    double* sQ = smem + S_TI * SREC;   // nj x QREC
    if (!dev::stage_two(sS, srec + (t1b + i0) * SREC, (uint32_t)(ni * SREC * 8), sQ, qrec + (t2b + j0) * QREC,
                        (uint32_t)(nj * QREC * 8), &bar, err))
        return;
    const int np = c_nbpts[order];
    for (int p = threadIdx.x; p < ni * nj; p += S_THREADS) {
        const int i = p / nj, j = p % nj;
        if (same && j0 + j < i0 + i) continue;
        const double* s = sS + i * SREC;
        const double* q = sQ + j * QREC;
        double acc = 0.0;
        for (int k = 0; k < np; ++k) acc += c_rules[order][k][3] * dev::operator_S(s, dev::ld3(q + 3 * k));
        const double val = q[48] * acc;
        const int64_t a = t1b + i0 + i, b = t2b + j0 + j;
        if (hm) {
            hm[lower_at(tpos[a], tpos[b], ld)] = val * coeff;
        } else {
            tmp[(i0 + i) * n2 + (j0 + j)] = val;
            if (same) tmp[(j0 + j) * n2 + (i0 + i)] = val;
        }
    }
}

void launch_S_block(const DevGeom& g, int64_t t1b, int64_t t1e, int64_t t2b, int64_t t2e, bool same, double coeff,
                    int order, double* hm, int64_t ld, double* tmp, int* err, cudaStream_t s) {
    const int64_t n1 = t1e - t1b, n2 = t2e - t2b;
    ProfScope prof_("s_block", s);
    dim3 grid(nblocks(n2, S_TJ), nblocks(n1, S_TI));
    const size_t sm = (size_t)(S_TI * SREC + S_TJ * QREC) * 8;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(s_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        attr = true;
    }
    s_block_kernel<<<grid, S_THREADS, sm, s>>>(g.srec, g.qrec, t1b, n1, t2b, n2, same ? 1 : 0, coeff, order, g.tpos,
                                               hm, ld, tmp, err);
    check_launch("S block");
}

// ---------------------------------------------------------------------------
// D block (BlocksBase::D operators.h:83-115): for t1 in A, t2 in B the three
// integrals over t1 of P1SingleLayerPotential(t2), stored per pair in a
// scratch array; the gather kernel below adds them into (t1, vertex) entries
// in a fixed order, so the result does not depend on thread timing.
// ---------------------------------------------------------------------------
constexpr int D_TI = 16, D_TJ = 32, D_THREADS = 256;

__global__ void __launch_bounds__(D_THREADS) d_block_kernel(const double* __restrict__ qrec,
                                                            const double* __restrict__ prec, int64_t tab, int64_t na,
                                                            int64_t tbb, int64_t nb, int order, double* tmp,
                                                            int* err) {
    extern __shared__ __align__(16) double smem[];
    __shared__ __align__(8) uint64_t bar;
    const int64_t i0 = (int64_t)blockIdx.y * D_TI, j0 = (int64_t)blockIdx.x * D_TJ;
    const int ni = (int)(na - i0 < (int64_t)D_TI ? na - i0 : (int64_t)D_TI), nj = (int)(nb - j0 < (int64_t)D_TJ ? nb - j0 : (int64_t)D_TJ);
    double* sQ = smem;                 // ni x QREC (integration triangles t1)
    double* sP = smem + D_TI * QREC;   // nj x PREC (analytic triangles t2)
    if (!dev::stage_two(sQ, qrec + (tab + i0) * QREC, (uint32_t)(ni * QREC * 8), sP, prec + (tbb + j0) * PREC,
                        (uint32_t)(nj * PREC * 8), &bar, err))
        return;
    const int np = c_nbpts[order];
    for (int p = threadIdx.x; p < ni * nj; p += D_THREADS) {
        const int i = p / nj, j = p % nj;
        const double* q = sQ + i * QREC;
        const double* P = sP + j * PREC;
        double acc[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < np; ++k) {
            double v[3];
            dev::p1_single_layer(P, dev::ld3(q + 3 * k), v);
            const double w = c_rules[order][k][3];
            acc[0] += w * v[0];
            acc[1] += w * v[1];
            acc[2] += w * v[2];
        }
        double* o = tmp + ((i0 + i) * nb + (j0 + j)) * 3;
        o[0] = q[48] * acc[0];
        o[1] = q[48] * acc[1];
        o[2] = q[48] * acc[2];
    }
}

void launch_D_block(const DevGeom& g, int64_t tab, int64_t tae, int64_t tbb, int64_t tbe, int order, double* tmp,
                    int* err, cudaStream_t s) {
    const int64_t na = tae - tab, nb = tbe - tbb;
    ProfScope prof_("d_block", s);
    dim3 grid(nblocks(nb, D_TJ), nblocks(na, D_TI));
    const size_t sm = (size_t)(D_TI * QREC + D_TJ * PREC) * 8;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(d_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        attr = true;
    }
    d_block_kernel<<<grid, D_THREADS, sm, s>>>(g.qrec, g.prec, tab, na, tbb, nb, order, tmp, err);
    check_launch("D block");
}

// HM(t1, v) += coeff * sum over triangles t2 of B containing v of tmp[t1][t2][local(v)]
// (the += of operators.h:108-109, in increasing t2 order).
__global__ void d_gather_kernel(int64_t tab, int64_t na, int64_t tbb, int64_t nb, int64_t vbb, int64_t nvb,
                                double coeff, const double* __restrict__ tmp, const int32_t* __restrict__ v2t_beg,
                                const int32_t* __restrict__ v2t_tri, const int8_t* __restrict__ v2t_loc,
                                const int32_t* __restrict__ tpos, int64_t nP, double* hm, int64_t ld, int rect) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= na * nvb) return;
    const int64_t iv = idx % nvb, ia = idx / nvb;
    const int64_t v = vbb + iv;
    double sum = 0.0;
    for (int k = v2t_beg[v]; k < v2t_beg[v + 1]; ++k) {
        const int64_t t2 = v2t_tri[k];
        if (t2 < tbb || t2 >= tbb + nb) continue;
        sum += tmp[(ia * nb + (t2 - tbb)) * 3 + v2t_loc[k]];
    }
    if (rect)   // rectangular output: row = the triangle's unknown, column = the vertex within B
        hm[tpos[tab + ia] + iv * ld] += coeff * sum;
    else
        hm[lower_at(tpos[tab + ia], nP + v, ld)] += coeff * sum;
}

void launch_D_gather(const DevGeom& g, int64_t tab, int64_t tae, int64_t tbb, int64_t tbe, int64_t vbb, int64_t vbe,
                     double coeff, const double* tmp, double* hm, int64_t ld, cudaStream_t s, bool rect) {
    ProfScope prof_("d_gather", s);
    const int64_t n = (tae - tab) * (vbe - vbb);
    d_gather_kernel<<<nblocks(n, 256), 256, 0, s>>>(tab, tae - tab, tbb, tbe - tbb, vbb, vbe - vbb, coeff, tmp,
                                                    g.v2t_beg, g.v2t_tri, g.v2t_loc, g.tpos, g.nP, hm, ld,
                                                    rect ? 1 : 0);
    check_launch("D gather");
}

// ---------------------------------------------------------------------------
// N block (BlocksBase::N operators.h:119-148 through DiagonalBlock::N :271-296
// and NonDiagonalBlock::N :454-480):
//   N(v1,v2) = - sum_{t1 ∋ v1, t2 ∋ v2} f (CB1.CB2) S(t1,t2) / (A1 A2)
// with f = 1/4 (1/2 for the same vertex across meshes).  S comes from the head
// matrix (scaled by coeff/Scoeff) or from a temporary unit-coefficient block.
// ---------------------------------------------------------------------------
__device__ __forceinline__ d3 edge_cb(const double* V, const int32_t* T, int64_t t, int loc) {
    // Edge(V) opposite the vertex: vertices {1,2},{2,0},{0,1} (triangle.h:87-94,154)
    const int a = (loc + 1) % 3, b = (loc + 2) % 3;
    return dev::ld3(V + 3 * (int64_t)T[3 * t + a]) - dev::ld3(V + 3 * (int64_t)T[3 * t + b]);
}

// Per vertex-triangle slot (CSR of v2t): q = CB / A, the edge vector opposite
// the vertex over the triangle's area (area from the OperatorS record).
__global__ void vertex_curls_kernel(int64_t nv, const int32_t* __restrict__ v2t_beg,
                                    const int32_t* __restrict__ v2t_tri, const int8_t* __restrict__ v2t_loc,
                                    const double* __restrict__ V, const int32_t* __restrict__ T,
                                    const double* __restrict__ srec, double* q) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nv) return;
    for (int k = v2t_beg[v]; k < v2t_beg[v + 1]; ++k) {
        const int64_t t = v2t_tri[k];
        const d3 cb = edge_cb(V, T, t, v2t_loc[k]);
        const double A = srec[t * SREC + 12];
        q[3 * (int64_t)k + 0] = cb.x / A;
        q[3 * (int64_t)k + 1] = cb.y / A;
        q[3 * (int64_t)k + 2] = cb.z / A;
    }
}

void launch_prepare_vertex_curls(const DevGeom& g, cudaStream_t s) {
    if (g.nv == 0) return;
    vertex_curls_kernel<<<nblocks(g.nv, 128), 128, 0, s>>>(g.nv, g.v2t_beg, g.v2t_tri, g.v2t_loc, g.V, g.T, g.srec,
                                                            g.v2t_q);
    check_launch("vertex curls");
}

// N block (operatorN, operators.h: the hypersingular operator by the curl
// identity): N(v1, v2) = -f sum_{a ni v1} sum_{b ni v2} (q_a(v1) . q_b(v2)) S(a, b),
// f = 1/4 (1/2 on a vertex shared by both sides of a non-self block), in two
// contractions with the sparse curl matrices instead of 36 curl products per
// vertex pair:
//   1. U_k(x, v) = sum_{y ni v} q_y,k(v) S(x, y), k = x, y, z, for every
//      triangle x of one side and vertex v of the other (x is the side along
//      which S is contiguous in memory: coalesced reads, warp-uniform loops);
//   2. N(vx, v) = -f sum_{x ni vx} sum_k q_x,k(vx) U_k(x, v).
// S(a, b) (a on mesh 1, b on mesh 2) is the block of the matrix (lower
// storage at the triangles' positions) or a dense a-major temporary.
__device__ __forceinline__ double n_block_s(const double* __restrict__ hm_src, int64_t ld,
                                            const double* __restrict__ tmp, int64_t nt2, const int32_t* __restrict__ tpos,
                                            int64_t t1b, int64_t t2b, int64_t a, int64_t b) {
    return hm_src ? hm_src[lower_at(tpos[a], tpos[b], ld)] : tmp[(a - t1b) * nt2 + (b - t2b)];
}

__global__ void n_curl_s_kernel(int64_t txb, int64_t nx, int64_t vyb, int64_t nvy, int64_t tyb, int64_t tye,
                                int swap, const double* __restrict__ hm_src, int64_t ld, const double* __restrict__ tmp,
                                int64_t nt2, int64_t t1b, int64_t t2b, const int32_t* __restrict__ v2t_beg,
                                const int32_t* __restrict__ v2t_tri, const double* __restrict__ vq,
                                const int32_t* __restrict__ tpos, double* __restrict__ U) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= nx * nvy) return;
    const int64_t ix = idx % nx, iv = idx / nx;   // x fastest
    const int64_t x = txb + ix, v = vyb + iv;
    double u0 = 0.0, u1 = 0.0, u2 = 0.0;
    for (int k = v2t_beg[v]; k < v2t_beg[v + 1]; ++k) {
        const int64_t y = v2t_tri[k];
        if (y < tyb || y >= tye) continue;
        const double sv = swap ? n_block_s(hm_src, ld, tmp, nt2, tpos, t1b, t2b, y, x)
                               : n_block_s(hm_src, ld, tmp, nt2, tpos, t1b, t2b, x, y);
        u0 = fma(vq[3 * (int64_t)k], sv, u0);
        u1 = fma(vq[3 * (int64_t)k + 1], sv, u1);
        u2 = fma(vq[3 * (int64_t)k + 2], sv, u2);
    }
    double* Uv = U + iv * 3 * nx + ix;
    Uv[0] = u0;
    Uv[nx] = u1;
    Uv[2 * nx] = u2;
}

__global__ void n_curl_u_kernel(int64_t vxb, int64_t nvx, int64_t txb, int64_t txe, int64_t vyb, int64_t nvy, int same,
                                int swap, double coeff, const double* __restrict__ U, int64_t nx,
                                const int32_t* __restrict__ v2t_beg, const int32_t* __restrict__ v2t_tri,
                                const double* __restrict__ vq, int64_t nP, double* hm, int64_t ld, int rect) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= nvx * nvy) return;
    const int64_t jx = idx % nvx, jy = idx / nvx;   // vx fastest
    const int64_t i1 = swap ? jy : jx, i2 = swap ? jx : jy;
    if (same && i2 > i1) return;
    const int64_t vx = vxb + jx, vy = vyb + jy;
    const int64_t v1 = swap ? vy : vx, v2 = swap ? vx : vy;
    const double factor = same ? 0.25 : (v1 == v2 ? 0.5 : 0.25);
    const double* Uy = U + jy * 3 * nx;
    double r = 0.0;
    for (int k = v2t_beg[vx]; k < v2t_beg[vx + 1]; ++k) {
        const int64_t x = v2t_tri[k];
        if (x < txb || x >= txe) continue;
        const int64_t ix = x - txb;
        r = fma(vq[3 * (int64_t)k], Uy[ix], r);
        r = fma(vq[3 * (int64_t)k + 1], Uy[nx + ix], r);
        r = fma(vq[3 * (int64_t)k + 2], Uy[2 * nx + ix], r);
    }
    const double result = -factor * r;
    if (rect)   // rectangular output: row = v1's unknown, column = v2 within its range
        hm[(nP + v1) + i2 * ld] += result * coeff;
    else
        hm[lower_at(nP + v1, nP + v2, ld)] += result * coeff;
}

void launch_N_block(const DevGeom& g, int64_t v1b, int64_t v1e, int64_t t1b, int64_t t1e, int64_t v2b, int64_t v2e,
                    int64_t t2b, int64_t t2e, bool same, double coeff, const double* hm_src, int64_t ld,
                    const double* tmp, double* hm, cudaStream_t s, bool rect, bool s_contiguous_b) {
    const int64_t n1 = v1e - v1b, n2 = v2e - v2b;
    if (n1 <= 0 || n2 <= 0) return;
    ProfScope prof_("n_block", s);
    // x: the triangles along which S is contiguous (b for a dense temporary, the later mesh in the matrix)
    const int swap = s_contiguous_b ? 1 : 0;
    const int64_t txb = swap ? t2b : t1b, txe = swap ? t2e : t1e, nx = txe - txb;
    const int64_t vxb = swap ? v2b : v1b, nvx = swap ? n2 : n1;
    const int64_t vyb = swap ? v1b : v2b, nvy = swap ? n1 : n2;
    const int64_t tyb = swap ? t1b : t2b, tye = swap ? t1e : t2e;
    DevBuf U((size_t)nx * nvy * 3 * sizeof(double), s);
    n_curl_s_kernel<<<nblocks(nx * nvy, 256), 256, 0, s>>>(txb, nx, vyb, nvy, tyb, tye, swap, hm_src, ld, tmp,
                                                           t2e - t2b, t1b, t2b, g.v2t_beg, g.v2t_tri, g.v2t_q, g.tpos,
                                                           U.as<double>());
    check_launch("N block (S by curls)");
    n_curl_u_kernel<<<nblocks(nvx * nvy, 256), 256, 0, s>>>(vxb, nvx, txb, txe, vyb, nvy, same ? 1 : 0, swap, coeff,
                                                            U.as<double>(), nx, g.v2t_beg, g.v2t_tri, g.v2t_q, g.nP,
                                                            hm, ld, rect ? 1 : 0);
    check_launch("N block");
}

// ---------------------------------------------------------------------------
// Deflation (Details::deflate, assembleHeadMat.cpp:27-60): add M(i0,i0)/n to
// every vertex pair of each outermost mesh.  The coefficient is read by a
// separate launch so no thread can observe a partially deflated diagonal.
// ---------------------------------------------------------------------------
__global__ void deflate_coef_kernel(const double* hm, int64_t pos, int64_t ld, double inv_nb, double* coef) {
    coef[0] = hm[pos + pos * ld] * inv_nb;
}
__global__ void deflate_add_kernel(int64_t vb, int64_t n, int64_t nP, const double* coef, double* hm, int64_t ld) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= n * n) return;
    const int64_t i1 = idx % n, i2 = idx / n;
    if (i2 > i1) return;
    hm[(nP + vb + i1) + (nP + vb + i2) * ld] += coef[0];
}

void launch_deflate(const DevGeom& g, const std::vector<std::pair<int64_t, int64_t>>& vranges, int64_t i_first,
                    int64_t nb, double* hm, int64_t ld, double* scratch, cudaStream_t s) {
    ProfScope prof_("deflate", s);
    const int64_t pos = g.nP + i_first;
    deflate_coef_kernel<<<1, 1, 0, s>>>(hm, pos, ld, 1.0 / (double)nb, scratch);
    check_launch("deflate coef");
    for (const auto& r : vranges) {
        const int64_t n = r.second - r.first;
        deflate_add_kernel<<<nblocks(n * n, 256), 256, 0, s>>>(r.first, n, g.nP, scratch, hm, ld);
        check_launch("deflate add");
    }
}

// ---------------------------------------------------------------------------
// Internal lower-triangle matrix -> reference numbering, dense (both halves)
// or SymMatrix packed upper.  ipos(r) = r >= nv ? r - nv : r + nP.
// ---------------------------------------------------------------------------
__global__ void to_reference_dense_kernel(int64_t N, int64_t nv, int64_t nP, const double* __restrict__ hm,
                                          int64_t ld, double* out, int64_t ldo) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= N) return;
    for (int64_t j = blockIdx.y; j < N; j += gridDim.y) {
        const int64_t a = i >= nv ? i - nv : i + nP, b = j >= nv ? j - nv : j + nP;
        out[i + j * ldo] = hm[lower_at(a, b, ld)];
    }
}
__global__ void to_reference_packed_kernel(int64_t N, int64_t nv, int64_t nP, const double* __restrict__ hm,
                                           int64_t ld, double* out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= N) return;
    for (int64_t j = blockIdx.y; j < N; j += gridDim.y) {
        if (i > j) continue;
        const int64_t a = i >= nv ? i - nv : i + nP, b = j >= nv ? j - nv : j + nP;
        out[i + j * (j + 1) / 2] = hm[lower_at(a, b, ld)];
    }
}

void launch_symmetrize_to_reference(const DevGeom& g, const double* hm_int, int64_t ld_int, double* out,
                                    int64_t ld_out, bool packed, cudaStream_t s) {
    ProfScope prof_("to_reference", s);
    dim3 grid(nblocks(g.Nref, 256), (unsigned)std::min<int64_t>(g.Nref, 32768));
    if (packed)
        to_reference_packed_kernel<<<grid, 256, 0, s>>>(g.Nref, g.nv, g.nP, hm_int, ld_int, out);
    else
        to_reference_dense_kernel<<<grid, 256, 0, s>>>(g.Nref, g.nv, g.nP, hm_int, ld_int, out, ld_out);
    check_launch("to reference");
}

// Rows of an internal-numbered N_int x ncol block (column-major, ldi) to the
// reference numbering [vertices | triangle unknowns], Nref x ncol (ldo).
__global__ void rows_to_reference_kernel(int64_t Nref, int64_t nv, int64_t nP, int64_t ncol,
                                         const double* __restrict__ in, int64_t ldi, double* out, int64_t ldo) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= Nref) return;
    const int64_t a = r < nv ? nP + r : r - nv;
    for (int64_t c = blockIdx.y; c < ncol; c += gridDim.y) out[r + c * ldo] = in[a + c * ldi];
}

void launch_rows_to_reference(const DevGeom& g, int64_t ncol, const double* in, int64_t ldi, double* out, int64_t ldo,
                              cudaStream_t s) {
    if (ncol <= 0 || g.Nref <= 0) return;
    dim3 grid(nblocks(g.Nref, 256), (unsigned)std::min<int64_t>(ncol, 32768));
    rows_to_reference_kernel<<<grid, 256, 0, s>>>(g.Nref, g.nv, g.nP, ncol, in, ldi, out, ldo);
    check_launch("rows to reference");
}

// Reference-numbered dense (lower triangle read) -> internal lower triangle,
// identity on the padding.
__global__ void from_reference_dense_kernel(int64_t N, int64_t nv, int64_t nP, int64_t nPt,
                                            const double* __restrict__ in, int64_t ldi, double* hm, int64_t ld) {
    const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;   // internal row
    if (a >= N) return;
    for (int64_t b = blockIdx.y; b <= a; b += gridDim.y) {             // internal column
        const bool pa = (a >= nPt && a < nP), pb = (b >= nPt && b < nP);
        if (pa || pb) {
            hm[a + b * ld] = (a == b) ? 1.0 : 0.0;
            continue;
        }
        const int64_t i = a < nPt ? a + nv : a - nP, j = b < nPt ? b + nv : b - nP;
        hm[a + b * ld] = i >= j ? in[i + j * ldi] : in[j + i * ldi];
    }
}

__global__ void pad_identity_kernel(int64_t nPt, int64_t nP, double* hm, int64_t ld) {
    const int64_t a = nPt + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (a < nP) hm[a + a * ld] = 1.0;
}

void launch_pad_identity(const DevGeom& g, double* hm, int64_t ld, cudaStream_t s) {
    if (g.nP == g.nPt) return;
    ProfScope prof_("pad_identity", s);
    pad_identity_kernel<<<1, 128, 0, s>>>(g.nPt, g.nP, hm, ld);
    check_launch("pad identity");
}

void launch_from_reference_dense(const DevGeom& g, const double* in, int64_t ldi, double* hm, int64_t ld,
                                 cudaStream_t s) {
    ProfScope prof_("from_reference", s);
    dim3 grid(nblocks(g.N, 256), (unsigned)std::min<int64_t>(g.N, 32768));
    from_reference_dense_kernel<<<grid, 256, 0, s>>>(g.N, g.nv, g.nP, g.nPt, in, ldi, hm, ld);
    check_launch("from reference");
}

// ===========================================================================
// Mixed-precision HeadMat assembly
//
// Far pairs (centroid distance >= rho_far x the larger max edge) are computed
// by a 16 x 16 Gauss product rule in FP32 -- the same outer rule as the
// reference, with the analytic inner integral replaced by the rule on the
// other triangle.  Coordinates are taken relative to each triangle's centroid
// and the centroid difference is formed in FP64 before rounding, so the FP32
// distances carry no cancellation.  One pass over a triangle pair yields S,
// D(t1 -> vertices of t2) and D(t2 -> vertices of t1): the 256 point-point
// distances are shared.  Near pairs are appended to a list and recomputed
// with the FP64 analytic kernels.
// ===========================================================================
// floats per triangle: centroid (3 doubles), 16-point offsets, normal, h, area (double), 7-point offsets,
// area (FP32)
constexpr int GREC = kFarRecFloats, GREC_P7 = 64, GREC_AF = GREC_P7 + 21;
// The 16-point rule of c_rules[3] rounded to FP32 (weights, barycentric nodes).
__constant__ __align__(8) float c_w16[16] = {0.144315607677786f, 0.095091634267284f, 0.095091634267284f, 0.095091634267284f, 0.032458497623198f, 0.032458497623198f, 0.032458497623198f, 0.103217370534718f, 0.103217370534718f, 0.103217370534718f, 0.027230314174434f, 0.027230314174434f, 0.027230314174434f, 0.027230314174434f, 0.027230314174434f, 0.027230314174434f};
__constant__ float c_b16[16][3] = {
    {0.333333333333333f, 0.333333333333333f, 0.333333333333333f},
    {0.081414823414554f, 0.459292588292722f, 0.459292588292722f},
    {0.459292588292722f, 0.081414823414554f, 0.459292588292722f},
    {0.459292588292722f, 0.459292588292722f, 0.081414823414554f},
    {0.898905543365937f, 0.050547228317031f, 0.050547228317031f},
    {0.050547228317031f, 0.898905543365937f, 0.050547228317031f},
    {0.050547228317031f, 0.050547228317031f, 0.898905543365937f},
    {0.658861384496479f, 0.170569307751760f, 0.170569307751761f},
    {0.170569307751760f, 0.658861384496479f, 0.170569307751761f},
    {0.170569307751760f, 0.170569307751761f, 0.658861384496479f},
    {0.008394777409957f, 0.728492392955404f, 0.263112829634639f},
    {0.728492392955404f, 0.008394777409957f, 0.263112829634639f},
    {0.728492392955404f, 0.263112829634639f, 0.008394777409957f},
    {0.008394777409957f, 0.263112829634639f, 0.728492392955404f},
    {0.263112829634639f, 0.008394777409957f, 0.728492392955404f},
    {0.263112829634639f, 0.728492392955404f, 0.008394777409957f}};
// The 7-point rule of c_rules[2] rounded to FP32, for well-separated pairs; weights padded with a zero eighth
// lane (the packed pair (6, 6) counts point 6 once).
__constant__ __align__(8) float c_w7[8] = {0.2250f, 0.132394152788506f, 0.132394152788506f, 0.132394152788506f,
                                           0.125939180544828f, 0.125939180544828f, 0.125939180544828f, 0.f};
__constant__ float c_b7[7][3] = {{0.333333333333333f, 0.333333333333333f, 0.333333333333333f},
                                 {0.470142064105115f, 0.470142064105115f, 0.059715871789770f},
                                 {0.470142064105115f, 0.059715871789770f, 0.470142064105115f},
                                 {0.059715871789770f, 0.470142064105115f, 0.470142064105115f},
                                 {0.101286507323456f, 0.101286507323456f, 0.797426985353088f},
                                 {0.101286507323456f, 0.797426985353088f, 0.101286507323456f},
                                 {0.797426985353088f, 0.101286507323456f, 0.101286507323456f}};


__global__ void prepare_gg_kernel(int64_t nt, const double* __restrict__ V, const int32_t* __restrict__ T,
                                  float* grec) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const d3 p0 = dev::ld3(V + 3 * (int64_t)T[3 * t]);
    const d3 p1 = dev::ld3(V + 3 * (int64_t)T[3 * t + 1]);
    const d3 p2 = dev::ld3(V + 3 * (int64_t)T[3 * t + 2]);
    const d3 c = (p0 + p1 + p2) * (1.0 / 3.0);
    float* g = grec + t * GREC;
    double* gc = reinterpret_cast<double*>(g);
    gc[0] = c.x; gc[1] = c.y; gc[2] = c.z;
    for (int k = 0; k < 16; ++k) {
        const d3 v = bary_point(c_rules[3][k], p0, p1, p2) - c;
        g[6 + 3 * k] = (float)v.x; g[7 + 3 * k] = (float)v.y; g[8 + 3 * k] = (float)v.z;
    }
    const d3 nn = dev::cross(p1 - p0, p2 - p0);
    const double nrm = dev::norm(nn);
    g[54] = (float)(nn.x / nrm); g[55] = (float)(nn.y / nrm); g[56] = (float)(nn.z / nrm);
    g[57] = (float)fmax(dev::norm(p1 - p0), fmax(dev::norm(p2 - p1), dev::norm(p0 - p2)));
    reinterpret_cast<double*>(g + 58)[0] = 0.5 * nrm;
    g[60] = g[61] = g[62] = g[63] = 0.f;
    for (int k = 0; k < 7; ++k) {
        const d3 v = bary_point(c_rules[2][k], p0, p1, p2) - c;
        g[GREC_P7 + 3 * k] = (float)v.x; g[GREC_P7 + 3 * k + 1] = (float)v.y; g[GREC_P7 + 3 * k + 2] = (float)v.z;
    }
    g[GREC_AF] = (float)(0.5 * nrm);
    for (int k = GREC_AF + 1; k < GREC; ++k) g[k] = 0.f;
}

void launch_prepare_gg(const DevGeom& g, float* grec, cudaStream_t s) {
    ProfScope prof_("prepare_gg", s);
    prepare_gg_kernel<<<nblocks(g.nt, 128), 128, 0, s>>>(g.nt, g.V, g.T, grec);
    check_launch("prepare_gg");
}

// Packed FP32 pairs (two lanes per 64-bit register) and the sm_100-family
// FP32x2 instructions on them: one issue slot performs two FP32 operations.
typedef unsigned long long f2;
__device__ __forceinline__ f2 pk2(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float lo2(f2 x) {
    float a, b;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x));
    return a;
}
__device__ __forceinline__ float hi2(f2 x) {
    float a, b;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x));
    return b;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// 1/sqrt(x) as the single approximate instruction (about 2 ulp, like rsqrtf);
// flushing denormals is harmless here: x is a squared distance between
// points of separated triangles.
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

constexpr int FF_TI = 128, FF_TJ = 16;
constexpr float kFarTier7 = 36.f;   // squared: pairs at >= 6 max edges take the 7-point rule

// One thread per t1 row, looping over the CTA's FF_TJ staged t2 records.
__global__ void __launch_bounds__(FF_TI, 3) ff_block_kernel(const float* __restrict__ grec, int64_t t1b, int64_t n1,
                                                         int64_t t2b, int64_t n2, int same, int wantS, int wantD12,
                                                         int wantD21, double cS, const int32_t* __restrict__ tpos,
                                                         double* hm, int64_t ld, double* stmp, double* d12,
                                                         double* d21, int2* near, int* near_count, int near_cap,
                                                         float rho, int* err) {
    __shared__ __align__(16) float sJ[FF_TJ * GREC];
    __shared__ __align__(8) uint64_t bar;
    const int64_t i0 = (int64_t)blockIdx.y * FF_TI, j0 = (int64_t)blockIdx.x * FF_TJ;
    if (same && j0 + FF_TJ <= i0) return;
    const int nj = (int)(n2 - j0 < (int64_t)FF_TJ ? n2 - j0 : (int64_t)FF_TJ);
    if (!dev::stage_two(sJ, grec + (t2b + j0) * GREC, (uint32_t)(nj * GREC * 4), nullptr, nullptr, 0, &bar, err))
        return;
    const int64_t i = i0 + threadIdx.x;
    if (i >= n1) return;
    const float* g1 = grec + (t1b + i) * GREC;
    const double* c1p = reinterpret_cast<const double*>(g1);
    const double c1x = c1p[0], c1y = c1p[1], c1z = c1p[2];
    const f2* W = reinterpret_cast<const f2*>(c_w16);   // weight pairs, read from the constant bank
    // t1's 7 points, packed (0,1) (2,3) (4,5) (6,6) (the last pair's second lane has a zero weight), held
    // across the loop: most pairs take the 7-point rule
    f2 Px[4], Py[4], Pz[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float* p7 = g1 + GREC_P7;
        const int u = 2 * k, v = 2 * k + 1 < 7 ? 2 * k + 1 : 6;
        Px[k] = pk2(p7[3 * u], p7[3 * v]);
        Py[k] = pk2(p7[3 * u + 1], p7[3 * v + 1]);
        Pz[k] = pk2(p7[3 * u + 2], p7[3 * v + 2]);
    }
    const float n1x = g1[54], n1y = g1[55], n1z = g1[56], h1 = g1[57];
    const float A1f = g1[GREC_AF], cSf = (float)cS;
    for (int jj = 0; jj < nj; ++jj) {
        const int64_t j = j0 + jj;
        if (same && j < i) continue;
        const float* g2 = sJ + jj * GREC;
        const double* c2p = reinterpret_cast<const double*>(g2);
        // the centroid difference in FP64 (no cancellation), rounded once; the rest of the pair in FP32
        const float fx = (float)(c2p[0] - c1x), fy = (float)(c2p[1] - c1y), fz = (float)(c2p[2] - c1z);
        const float hmax = fmaxf(h1, g2[57]);
        const float dist2 = fmaf(fx, fx, fmaf(fy, fy, fz * fz));
        if (dist2 < rho * rho * hmax * hmax) {
            const int slot = atomicAdd(near_count, 1);
            if (slot < near_cap) near[slot] = make_int2((int)i, (int)j);
            continue;
        }
        const float n2x = g2[54], n2y = g2[55], n2z = g2[56];
        // r = d + Q_q - P_k (d: centroid difference, P_k / Q_q: the points' offsets in the planes of t1 / t2,
        // so P_k . n1 = Q_q . n2 = 0): r . n2 = d . n2 - P_k . n2 depends on k only and r . n1 = d . n1 + Q_q . n1
        // on q only, folded into the weights: WD[k] = w_k (r . n2), cq = -w_q (r . n1)
        const float dn2 = fmaf(fx, n2x, fmaf(fy, n2y, fz * n2z));
        const float dn1 = fmaf(fx, n1x, fmaf(fy, n1y, fz * n1z));
        const f2 DN2 = pk2(dn2, dn2), N2x = pk2(n2x, n2x), N2y = pk2(n2y, n2y), N2z = pk2(n2z, n2z);
        float s = 0.f, e0 = 0.f, e1 = 0.f, e2 = 0.f, u0 = 0.f, u1 = 0.f, u2 = 0.f;   // u: D21
        if (dist2 >= kFarTier7 * hmax * hmax) {
            // well separated (>= 6 max edges): the 7 x 7 product rule, within 1e-7 of the 16 x 16 one there
            const f2* W7 = reinterpret_cast<const f2*>(c_w7);
            f2 WD7[4], A7[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                WD7[k] = mul2(W7[k], sub2(DN2, fma2(Px[k], N2x, fma2(Py[k], N2y, mul2(Pz[k], N2z)))));
                A7[k] = pk2(0.f, 0.f);
            }
            const float* q7 = g2 + GREC_P7;
#pragma unroll
            for (int q = 0; q < 7; ++q) {
                const float qx = q7[3 * q], qy = q7[3 * q + 1], qz = q7[3 * q + 2];
                const float wq = c_w7[q];
                const float cq = -wq * (dn1 + fmaf(qx, n1x, fmaf(qy, n1y, qz * n1z)));
                const f2 Yx = pk2(fx + qx, fx + qx), Yy = pk2(fy + qy, fy + qy), Yz = pk2(fz + qz, fz + qz),
                         CQ = pk2(cq, cq);
                f2 SQ = pk2(0.f, 0.f), K12 = pk2(0.f, 0.f);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const f2 rx = sub2(Yx, Px[k]), ry = sub2(Yy, Py[k]), rz = sub2(Yz, Pz[k]);
                    const f2 r2 = fma2(rx, rx, fma2(ry, ry, mul2(rz, rz)));
                    const f2 ir = pk2(rsqrt_ftz(lo2(r2)), rsqrt_ftz(hi2(r2)));
                    const f2 ir3 = mul2(mul2(ir, ir), ir);
                    SQ = fma2(W7[k], ir, SQ);
                    K12 = fma2(WD7[k], ir3, K12);
                    A7[k] = fma2(CQ, ir3, A7[k]);
                }
                s = fmaf(wq, lo2(SQ) + hi2(SQ), s);
                const float kq = wq * (lo2(K12) + hi2(K12));
                e0 = fmaf(kq, c_b7[q][0], e0);
                e1 = fmaf(kq, c_b7[q][1], e1);
                e2 = fmaf(kq, c_b7[q][2], e2);
            }
            if (wantD21 || (same && wantD12)) {
#pragma unroll
                for (int p = 0; p < 7; ++p) {
                    const float a = c_w7[p] * ((p & 1) ? hi2(A7[p / 2]) : lo2(A7[p / 2]));
                    u0 = fmaf(a, c_b7[p][0], u0);
                    u1 = fmaf(a, c_b7[p][1], u1);
                    u2 = fmaf(a, c_b7[p][2], u2);
                }
            }
        } else {
            // the 16 points of t1 in packed pairs (even p in the low lane, odd p in the high lane; the inner
            // products run two point pairs per FP32x2 instruction), loaded (L1) for the few pairs of this tier
            // instead of held across the loop: the registers go to more resident warps
            f2 P1x[8], P1y[8], P1z[8], WD[8], A21[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                P1x[k] = pk2(g1[6 + 6 * k], g1[9 + 6 * k]);
                P1y[k] = pk2(g1[7 + 6 * k], g1[10 + 6 * k]);
                P1z[k] = pk2(g1[8 + 6 * k], g1[11 + 6 * k]);
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                WD[k] = mul2(W[k], sub2(DN2, fma2(P1x[k], N2x, fma2(P1y[k], N2y, mul2(P1z[k], N2z)))));
                A21[k] = pk2(0.f, 0.f);
            }
            for (int q = 0; q < 16; ++q) {
                const float qx = g2[6 + 3 * q], qy = g2[7 + 3 * q], qz = g2[8 + 3 * q];
                const float yx = fx + qx, yy = fy + qy, yz = fz + qz;
                const float wq = c_w16[q];
                const float cq = -wq * (dn1 + fmaf(qx, n1x, fmaf(qy, n1y, qz * n1z)));
                const f2 Yx = pk2(yx, yx), Yy = pk2(yy, yy), Yz = pk2(yz, yz), CQ = pk2(cq, cq);
                f2 SQ = pk2(0.f, 0.f), K12 = pk2(0.f, 0.f);
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const f2 rx = sub2(Yx, P1x[k]), ry = sub2(Yy, P1y[k]), rz = sub2(Yz, P1z[k]);
                    const f2 r2 = fma2(rx, rx, fma2(ry, ry, mul2(rz, rz)));
                    const f2 ir = pk2(rsqrt_ftz(lo2(r2)), rsqrt_ftz(hi2(r2)));
                    const f2 ir3 = mul2(mul2(ir, ir), ir);
                    SQ = fma2(W[k], ir, SQ);
                    K12 = fma2(WD[k], ir3, K12);
                    A21[k] = fma2(CQ, ir3, A21[k]);
                }
                s = fmaf(wq, lo2(SQ) + hi2(SQ), s);
                const float kq = wq * (lo2(K12) + hi2(K12));
                e0 = fmaf(kq, c_b16[q][0], e0);
                e1 = fmaf(kq, c_b16[q][1], e1);
                e2 = fmaf(kq, c_b16[q][2], e2);
            }
            if (wantD21 || (same && wantD12)) {
#pragma unroll
                for (int p = 0; p < 16; ++p) {
                    const float a = c_w16[p] * ((p & 1) ? hi2(A21[p / 2]) : lo2(A21[p / 2]));
                    u0 = fmaf(a, c_b16[p][0], u0);
                    u1 = fmaf(a, c_b16[p][1], u1);
                    u2 = fmaf(a, c_b16[p][2], u2);
                }
            }
        }
        // the sums are FP32: scaled by the area product in FP32, widened once each
        const float AA = A1f * g2[GREC_AF];
        if (wantS) {
            if (hm)
                hm[lower_at(tpos[t1b + i], tpos[t2b + j], ld)] = (double)(s * (AA * cSf));
            else {
                stmp[i * n2 + j] = (double)(s * AA);
                if (same) stmp[j * n2 + i] = (double)(s * AA);
            }
        }
        if (wantD12) {
            double* o = d12 + (i * n2 + j) * 3;
            o[0] = (double)(e0 * AA); o[1] = (double)(e1 * AA); o[2] = (double)(e2 * AA);
        }
        if (wantD21 || (same && wantD12)) {
            double* o = same ? d12 + (j * n2 + i) * 3 : d21 + (j * n1 + i) * 3;
            o[0] = (double)(u0 * AA); o[1] = (double)(u1 * AA); o[2] = (double)(u2 * AA);
        }
    }
}

// Near pairs: the FP64 analytic kernels of the reference (same outer rule).
// One lane per (pair, point of the rule): 16 lanes hold a pair, each lane
// evaluates the analytic integrals at its point (S and D21 over t1 at the
// points of t2, with shared distances and solid angle; D12 over t2 at the
// points of t1) and the weighted values are summed across the 16 lanes by
// shuffles.  Short per-thread chains and many warps hide the latency of the
// FP64 transcendentals.
constexpr int NP_LANES = 16;

__global__ void __launch_bounds__(128) near_pairs_kernel(
    const int2* __restrict__ near, int count, const double* __restrict__ srec, const double* __restrict__ prec,
    const double* __restrict__ qrec, int64_t t1b, int64_t n1, int64_t t2b, int64_t n2, int same, int wantS,
    int wantD12, int wantD21, double cS, int order, const int32_t* __restrict__ tpos, double* hm, int64_t ld,
    double* stmp, double* d12, double* d21) {
    const int64_t g = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / NP_LANES;   // pair
    const int m = threadIdx.x % NP_LANES;                                            // point of the rule
    const bool live = g < count;   // every lane takes part in the shuffles
    int64_t i = 0, j = 0;
    if (live) {
        i = near[g].x;
        j = near[g].y;
    }
    const int64_t a = t1b + i, b = t2b + j;
    const bool wantP = (wantD21 || (same && wantD12)) && !(same && i == j);
    double sv = 0.0, p[3] = {0, 0, 0}, e[3] = {0, 0, 0};
    if (live && m < c_nbpts[order]) {
        const double w = c_rules[order][m][3];
        if (wantS || wantP) {
            const d3 x2 = dev::ld3(qrec + b * QREC + 3 * m);
            double v[3] = {0, 0, 0};
            if (wantS && wantP)
                sv = w * dev::operator_S_p1(srec + a * SREC, prec + a * PREC, x2, v);
            else if (wantS)
                sv = w * dev::operator_S(srec + a * SREC, x2);
            else
                dev::p1_single_layer(prec + a * PREC, x2, v);
            p[0] = w * v[0]; p[1] = w * v[1]; p[2] = w * v[2];
        }
        if (wantD12) {   // integral over t1 of P1SLP(t2)
            double v[3];
            dev::p1_single_layer(prec + b * PREC, dev::ld3(qrec + a * QREC + 3 * m), v);
            e[0] = w * v[0]; e[1] = w * v[1]; e[2] = w * v[2];
        }
    }
#pragma unroll
    for (int o = NP_LANES / 2; o > 0; o >>= 1) {
        sv += __shfl_xor_sync(0xffffffffu, sv, o);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            p[c] += __shfl_xor_sync(0xffffffffu, p[c], o);
            e[c] += __shfl_xor_sync(0xffffffffu, e[c], o);
        }
    }
    if (!live || m != 0) return;
    if (wantS) {
        const double val = qrec[b * QREC + 48] * sv;
        if (hm)
            hm[lower_at(tpos[a], tpos[b], ld)] = val * cS;
        else {
            stmp[i * n2 + j] = val;
            if (same) stmp[j * n2 + i] = val;
        }
    }
    if (wantD12) {
        const double A = qrec[a * QREC + 48];
        double* o = d12 + (i * n2 + j) * 3;
        o[0] = A * e[0]; o[1] = A * e[1]; o[2] = A * e[2];
    }
    if (wantP) {
        const double A = qrec[b * QREC + 48];
        double* o = same ? d12 + (j * n2 + i) * 3 : d21 + (j * n1 + i) * 3;
        o[0] = A * p[0]; o[1] = A * p[1]; o[2] = A * p[2];
    }
}

void launch_ff_block(const DevGeom& g, const float* grec, int64_t t1b, int64_t t1e, int64_t t2b, int64_t t2e,
                     bool same, bool wantS, bool wantD12, bool wantD21, double cS, double* hm, int64_t ld,
                     double* stmp, double* d12, double* d21, int2* near, int* near_count, int near_cap, float rho,
                     int* err, cudaStream_t s) {
    ProfScope prof_("ff_block", s);
    const int64_t n1 = t1e - t1b, n2 = t2e - t2b;
    dim3 grid(nblocks(n2, FF_TJ), nblocks(n1, FF_TI));
    ff_block_kernel<<<grid, FF_TI, 0, s>>>(grec, t1b, n1, t2b, n2, same ? 1 : 0, wantS ? 1 : 0, wantD12 ? 1 : 0,
                                           wantD21 ? 1 : 0, cS, g.tpos, hm, ld, stmp, d12, d21, near, near_count,
                                           near_cap, rho, err);
    check_launch("ff block");
}

void launch_near_pairs(const DevGeom& g, const int2* near, int count, int64_t t1b, int64_t t1e, int64_t t2b,
                       int64_t t2e, bool same, bool wantS, bool wantD12, bool wantD21, double cS, int order,
                       double* hm, int64_t ld, double* stmp, double* d12, double* d21, cudaStream_t s) {
    if (count <= 0) return;
    if (order < 0 || order > 3) throw Error(OMG_ERR_INVALID, "near pairs: rule of more than 16 points");
    ProfScope prof_("near_pairs", s);
    near_pairs_kernel<<<nblocks((int64_t)count * NP_LANES, 128), 128, 0, s>>>(near, count, g.srec, g.prec, g.qrec,
                                                                              t1b, t1e - t1b, t2b,
                                                          t2e - t2b, same ? 1 : 0, wantS ? 1 : 0, wantD12 ? 1 : 0,
                                                          wantD21 ? 1 : 0, cS, order, g.tpos, hm, ld, stmp, d12, d21);
    check_launch("near pairs");
}

// ===========================================================================
// Sources and sensors
// ===========================================================================

// Interface::contains (OpenMEEG/src/interface.cpp:18-35) on an oriented solid angle.
__device__ __forceinline__ bool almost_eq(double x, double y) {
    return fabs(x - y) < 2.220446049250313e-16 * fabs(x + y) * 1e3 || fabs(x - y) < 2.2250738585072014e-308;
}
__device__ __forceinline__ bool interface_contains(double s) {
    const double fourpi = 12.566370614359172;
    if (almost_eq(s, -fourpi)) return true;
    if (almost_eq(s, 0.0)) return false;
    if (almost_eq(s, fourpi)) return true;
    return fabs(s) > 0.5 * fourpi;
}

// Mesh::solid_angle (mesh.cpp:239-244) of every mesh seen from every point:
// one CTA per point, a fixed-order tree reduction per mesh.
__global__ void mesh_solid_angles_kernel(const double* __restrict__ pts, int64_t pstride, int nmesh,
                                         const int64_t* __restrict__ tbeg, const double* __restrict__ srec,
                                         double* out) {
    __shared__ double red[256];
    const int64_t i = blockIdx.x;
    const d3 p = dev::ld3(pts + i * pstride);
    for (int m = 0; m < nmesh; ++m) {
        double acc = 0.0;
        for (int64_t t = tbeg[m] + threadIdx.x; t < tbeg[m + 1]; t += blockDim.x) {
            const double* s = srec + t * SREC;
            const d3 r0 = dev::ld3(s) - p, r1 = dev::ld3(s + 3) - p, r2 = dev::ld3(s + 6) - p;
            acc += dev::solid_angle(r0, r1, r2, dev::norm(r0), dev::norm(r1), dev::norm(r2), dev::ld3(s + 9), s[12]);
        }
        red[threadIdx.x] = acc;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[i * nmesh + m] = red[0];
        __syncthreads();
    }
}

// Same, screened in FP32 for the domain lookup of the mixed path: a closed
// mesh subtends 0 or +-4 pi, so only the classification |sum| > 2 pi matters;
// a sum within 1 of 2 pi (a point at the surface, where FP32 could tip the
// test) is recomputed in FP64, so the domains are those of the FP64 sums.
__global__ void mesh_solid_angles_screened_kernel(const double* __restrict__ pts, int64_t pstride, int nmesh,
                                                  const int64_t* __restrict__ tbeg, const double* __restrict__ srec,
                                                  double* out) {
    __shared__ float redf[256];
    __shared__ double red[256];
    const int64_t i = blockIdx.x;
    const d3 p = dev::ld3(pts + i * pstride);
    for (int m = 0; m < nmesh; ++m) {
        float acc = 0.f;
        for (int64_t t = tbeg[m] + threadIdx.x; t < tbeg[m + 1]; t += blockDim.x) {
            const double* s = srec + t * SREC;
            const float ax = (float)(s[0] - p.x), ay = (float)(s[1] - p.y), az = (float)(s[2] - p.z);
            const float bx = (float)(s[3] - p.x), by = (float)(s[4] - p.y), bz = (float)(s[5] - p.z);
            const float cx = (float)(s[6] - p.x), cy = (float)(s[7] - p.y), cz = (float)(s[8] - p.z);
            const float da = sqrtf(ax * ax + ay * ay + az * az), db = sqrtf(bx * bx + by * by + bz * bz),
                        dc = sqrtf(cx * cx + cy * cy + cz * cz);
            const float num = 2.f * (float)s[12] * (ax * (float)s[9] + ay * (float)s[10] + az * (float)s[11]);
            const float den = da * db * dc + da * (bx * cx + by * cy + bz * cz) + db * (cx * ax + cy * ay + cz * az) +
                              dc * (ax * bx + ay * by + az * bz);
            acc += 2.f * atan2f(num, den);
        }
        redf[threadIdx.x] = acc;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) redf[threadIdx.x] += redf[threadIdx.x + w];
            __syncthreads();
        }
        const float sum = redf[0];
        __syncthreads();
        if (fabsf(fabsf(sum) - 6.2831853f) > 1.f && sum == sum) {   // clear of the 2 pi boundary
            if (threadIdx.x == 0) out[i * nmesh + m] = fabsf(sum) < 3.1415927f ? 0.0 : (sum > 0 ? 1.0 : -1.0) *
                                                                                          12.566370614359172;
            continue;
        }
        double accd = 0.0;   // near the surface: the FP64 sum of the reference formula
        for (int64_t t = tbeg[m] + threadIdx.x; t < tbeg[m + 1]; t += blockDim.x) {
            const double* s = srec + t * SREC;
            const d3 r0 = dev::ld3(s) - p, r1 = dev::ld3(s + 3) - p, r2 = dev::ld3(s + 6) - p;
            accd += dev::solid_angle(r0, r1, r2, dev::norm(r0), dev::norm(r1), dev::norm(r2), dev::ld3(s + 9), s[12]);
        }
        red[threadIdx.x] = accd;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[i * nmesh + m] = red[0];
        __syncthreads();
    }
}

// Geometry::domain(point) (geometry.cpp:146-154, domain.cpp:12-17): the first
// domain all of whose boundaries agree with the point's inside/outside state.
// A boundary is an interface: the solid angles of its meshes are summed with
// their orientations (Interface::solid_angle, interface.cpp:40-45); the
// domain's per-mesh entries of one interface share a group index.
__global__ void domain_lookup_kernel(int64_t n, int nmesh, const double* __restrict__ sa, int ndom, int maxb,
                                     const int* __restrict__ dnb, const int* __restrict__ bmesh,
                                     const int* __restrict__ binside, const int* __restrict__ borient,
                                     const int* __restrict__ bgrp, int forced, int* dom, int* err) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (forced >= 0) {
        dom[i] = forced;
        return;
    }
    int found = -1;
    for (int d = 0; d < ndom && found < 0; ++d) {
        bool ok = true;
        double acc = 0.0;
        for (int k = 0; k < dnb[d]; ++k) {
            const int q = d * maxb + k;
            acc += borient[q] * sa[i * nmesh + bmesh[q]];
            if (k + 1 == dnb[d] || bgrp[q + 1] != bgrp[q]) {   // end of this interface's meshes
                if (interface_contains(acc) != (binside[q] != 0)) ok = false;
                acc = 0.0;
            }
        }
        if (ok) found = d;
    }
    dom[i] = found;
    if (found < 0) atomicExch(err, -1 /* OMG_ERR_INVALID: point in no domain */);
}

// Integrands of the DipSourceMat: Dipole::potential / Dipole::gradient
// (dipole.h:29-46) and the barycentric weights of PotentialDerivative
// (analytics.h:140-150, BarycentricCoordinates.h:33-69).
struct DsmTri {
    d3 p0, e10, e20, n;
    double d11, d12, d22;
};
__device__ __forceinline__ void dsm_eval(int kind, const DsmTri& T, d3 r0, d3 q, d3 r, double out[3]) {
    const d3 x = r - r0;
    if (kind == 1) {
        const double nrm2 = dev::dot(x, x);
        out[0] = dev::dot(q, x) / (nrm2 * sqrt(nrm2));
        return;
    }
    const double inv = 1.0 / dev::dot(x, x);
    const d3 grad = q - x * (3 * dev::dot(q, x) * inv);
    const double g = dev::dot(grad, T.n) * (inv * sqrt(inv));
    const d3 v = r - T.p0;
    const double a1 = dev::dot(v, T.e10), a2 = dev::dot(v, T.e20);
    const double l1 = T.d11 * a1 + T.d12 * a2;
    const double l2 = T.d12 * a1 + T.d22 * a2;
    const double l0 = 1.0 - l1 - l2;
    out[0] = g * l0;
    out[1] = g * l1;
    out[2] = g * l2;
}

__device__ __forceinline__ void dsm_rule(int kind, int order, const DsmTri& T, d3 r0, d3 q, d3 P0, d3 P1, d3 P2,
                                         double area, double res[3]) {
    double acc[3] = {0.0, 0.0, 0.0};
    const int np = c_nbpts[order];
    for (int k = 0; k < np; ++k) {
        const d3 x = bary_point(c_rules[order][k], P0, P1, P2);
        double v[3];
        dsm_eval(kind, T, r0, q, x, v);
        const double w = c_rules[order][k][3];
        acc[0] += w * v[0];
        if (kind == 0) {
            acc[1] += w * v[1];
            acc[2] += w * v[2];
        }
    }
    res[0] = area * acc[0];
    res[1] = area * acc[1];
    res[2] = area * acc[2];
}

__device__ __forceinline__ void subtriangle(d3& P0, d3& P1, d3& P2, int c) {
    const d3 m0 = (P1 + P2) * 0.5, m1 = (P2 + P0) * 0.5, m2 = (P0 + P1) * 0.5;
    if (c == 0) { P1 = m1; P2 = m2; }
    else if (c == 1) { P0 = m0; P2 = m2; }
    else if (c == 2) { P0 = m0; P1 = m1; }
    else { P0 = m0; P1 = m1; P2 = m2; }
}

constexpr int DSM_MAX_LEVELS = 12;
constexpr int DSM_STACK = 3 * (DSM_MAX_LEVELS + 1) + 4;

// Integrator::integrate with adaptive_integration (integrator.h:44-48,228-252)
// as an explicit depth-first stack.  A node is its path of child indices from
// the root (2 bits per level), so the stack holds no vertex coordinates.
__device__ void dsm_adaptive(int kind, int order, int levels, double tol, const DsmTri& T, d3 r0, d3 q, d3 R0, d3 R1,
                             d3 R2, double area, double result[3]) {
    double coarse[3];
    dsm_rule(kind, order, T, r0, q, R0, R1, R2, area, coarse);
    if (levels == 0) {
        result[0] = coarse[0]; result[1] = coarse[1]; result[2] = coarse[2];
        return;
    }
    uint32_t st_path[DSM_STACK];
    int8_t st_depth[DSM_STACK], st_level[DSM_STACK];
    double st_c[DSM_STACK][3];
    int sp = 0;
    st_path[0] = 0; st_depth[0] = 0; st_level[0] = (int8_t)levels;
    st_c[0][0] = coarse[0]; st_c[0][1] = coarse[1]; st_c[0][2] = coarse[2];
    sp = 1;
    double total[3] = {0.0, 0.0, 0.0};
    const int dim = kind == 0 ? 3 : 1;
    while (sp > 0) {
        --sp;
        const uint32_t path = st_path[sp];
        const int depth = st_depth[sp], level = st_level[sp];
        const double c0 = st_c[sp][0], c1 = st_c[sp][1], c2 = st_c[sp][2];
        d3 P0 = R0, P1 = R1, P2 = R2;
        double a = area;
        for (int d = 0; d < depth; ++d) {
            subtriangle(P0, P1, P2, (path >> (2 * d)) & 3);
            a *= 0.25;
        }
        const double sub = 0.25 * a;
        double integ[4][3];
        double ref[3] = {0.0, 0.0, 0.0};
        for (int c = 0; c < 4; ++c) {
            d3 Q0 = P0, Q1 = P1, Q2 = P2;
            subtriangle(Q0, Q1, Q2, c);
            dsm_rule(kind, order, T, r0, q, Q0, Q1, Q2, sub, integ[c]);
            for (int k = 0; k < dim; ++k) ref[k] += integ[c][k];
        }
        double dn, cn;
        if (dim == 1) {
            dn = fabs(c0 - ref[0]);
            cn = fabs(c0);
        } else {
            const double e0 = c0 - ref[0], e1 = c1 - ref[1], e2 = c2 - ref[2];
            dn = sqrt(e0 * e0 + e1 * e1 + e2 * e2);
            cn = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
        }
        if (dn <= tol * cn || level == 0) {
            for (int k = 0; k < dim; ++k) total[k] += ref[k];
            continue;
        }
        for (int c = 3; c >= 0; --c) {
            st_path[sp] = path | ((uint32_t)c << (2 * depth));
            st_depth[sp] = (int8_t)(depth + 1);
            st_level[sp] = (int8_t)(level - 1);
            st_c[sp][0] = integ[c][0]; st_c[sp][1] = integ[c][1]; st_c[sp][2] = integ[c][2];
            ++sp;
        }
    }
    result[0] = total[0]; result[1] = total[1]; result[2] = total[2];
}

// The same integration by a group of four lanes (lanes 4 g .. 4 g + 3 of a
// warp, `mask` their bits): each node's four children are integrated one per
// lane, each child's rule summed in the order of dsm_rule, and the values are
// exchanged by shuffles, so every refinement decision and every sum is the
// one of dsm_adaptive; the four lanes run the same control flow.
__device__ void dsm_adaptive_g4(int kind, int order, int levels, double tol, const DsmTri& T, d3 r0, d3 q, d3 R0,
                                d3 R1, d3 R2, double area, double result[3], unsigned mask, int lane4) {
    double coarse[3];
    dsm_rule(kind, order, T, r0, q, R0, R1, R2, area, coarse);
    if (levels == 0) {
        result[0] = coarse[0]; result[1] = coarse[1]; result[2] = coarse[2];
        return;
    }
    const int base = (threadIdx.x & 31) & ~3;
    uint32_t st_path[DSM_STACK];
    int8_t st_depth[DSM_STACK], st_level[DSM_STACK];
    double st_c[DSM_STACK][3];
    int sp = 0;
    st_path[0] = 0; st_depth[0] = 0; st_level[0] = (int8_t)levels;
    st_c[0][0] = coarse[0]; st_c[0][1] = coarse[1]; st_c[0][2] = coarse[2];
    sp = 1;
    double total[3] = {0.0, 0.0, 0.0};
    const int dim = kind == 0 ? 3 : 1;
    while (sp > 0) {
        --sp;
        const uint32_t path = st_path[sp];
        const int depth = st_depth[sp], level = st_level[sp];
        const double c0 = st_c[sp][0], c1 = st_c[sp][1], c2 = st_c[sp][2];
        d3 P0 = R0, P1 = R1, P2 = R2;
        double a = area;
        for (int d = 0; d < depth; ++d) {
            subtriangle(P0, P1, P2, (path >> (2 * d)) & 3);
            a *= 0.25;
        }
        const double sub = 0.25 * a;
        double mine[3];
        {
            d3 Q0 = P0, Q1 = P1, Q2 = P2;
            subtriangle(Q0, Q1, Q2, lane4);
            dsm_rule(kind, order, T, r0, q, Q0, Q1, Q2, sub, mine);
        }
        double integ[4][3];
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
            for (int k = 0; k < 3; ++k) integ[c][k] = __shfl_sync(mask, mine[k], base + c);
        double ref[3] = {0.0, 0.0, 0.0};
        for (int c = 0; c < 4; ++c)
            for (int k = 0; k < dim; ++k) ref[k] += integ[c][k];
        double dn, cn;
        if (dim == 1) {
            dn = fabs(c0 - ref[0]);
            cn = fabs(c0);
        } else {
            const double e0 = c0 - ref[0], e1 = c1 - ref[1], e2 = c2 - ref[2];
            dn = sqrt(e0 * e0 + e1 * e1 + e2 * e2);
            cn = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
        }
        if (dn <= tol * cn || level == 0) {
            for (int k = 0; k < dim; ++k) total[k] += ref[k];
            continue;
        }
        for (int c = 3; c >= 0; --c) {
            st_path[sp] = path | ((uint32_t)c << (2 * depth));
            st_depth[sp] = (int8_t)(depth + 1);
            st_level[sp] = (int8_t)(level - 1);
            st_c[sp][0] = integ[c][0]; st_c[sp][1] = integ[c][1]; st_c[sp][2] = integ[c][2];
            ++sp;
        }
    }
    result[0] = total[0]; result[1] = total[1]; result[2] = total[2];
}


// Mixed precision: the first adaptive level in FP32 with coordinates relative
// to the triangle centroid.  The FP32 value is kept only when the acceptance
// test |coarse - refined| <= tol |coarse| (integrator.h:245) holds with a
// factor-2 margin -- a decision FP32 rounding cannot flip; otherwise the
// caller recomputes in FP64.
struct DsmTriF {
    float3 p0, e10, e20, n;   // p0 relative to the centroid
    float d11, d12, d22;
};
__device__ __forceinline__ float3 fmid(float3 a, float3 b) {
    return make_float3(0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z));
}
// Both integrands of the first level at once, sharing the point's distance:
// out[0..2] the kind-0 values (P1-weighted normal derivative), out[3] the
// kind-1 value (potential); the expressions of the separate evaluations.
__device__ __forceinline__ void dsm_eval2_f(const DsmTriF& T, float3 xc, float3 q, float3 v, float out[4]) {
    const float3 x = make_float3(xc.x + v.x, xc.y + v.y, xc.z + v.z);   // r - r0
    const float n2 = x.x * x.x + x.y * x.y + x.z * x.z;
    const float qx = q.x * x.x + q.y * x.y + q.z * x.z;
    out[3] = qx / (n2 * sqrtf(n2));
    const float inv = 1.f / n2;
    const float3 g = make_float3(q.x - 3.f * qx * x.x * inv, q.y - 3.f * qx * x.y * inv, q.z - 3.f * qx * x.z * inv);
    const float gn = (g.x * T.n.x + g.y * T.n.y + g.z * T.n.z) * (inv * sqrtf(inv));
    const float3 w = make_float3(v.x - T.p0.x, v.y - T.p0.y, v.z - T.p0.z);   // r - p0
    const float a1 = w.x * T.e10.x + w.y * T.e10.y + w.z * T.e10.z;
    const float a2 = w.x * T.e20.x + w.y * T.e20.y + w.z * T.e20.z;
    const float l1 = T.d11 * a1 + T.d12 * a2, l2 = T.d12 * a1 + T.d22 * a2;
    out[0] = gn * (1.f - l1 - l2);
    out[1] = gn * l1;
    out[2] = gn * l2;
}
__device__ __forceinline__ void dsm_rule2_f(const DsmTriF& T, float3 xc, float3 q, float3 P0, float3 P1, float3 P2,
                                            float area, float res[4]) {
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
    for (int k = 0; k < 16; ++k) {
        const float b0 = c_b16[k][0], b1 = c_b16[k][1], b2 = c_b16[k][2];
        const float3 v = make_float3(b0 * P0.x + b1 * P1.x + b2 * P2.x, b0 * P0.y + b1 * P1.y + b2 * P2.y,
                                     b0 * P0.z + b1 * P1.z + b2 * P2.z);
        float e[4];
        dsm_eval2_f(T, xc, q, v, e);
        const float w = c_w16[k];
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[c] = fmaf(w, e[c], acc[c]);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) res[c] = area * acc[c];
}
// The first adaptive level of both integrals in one pass over the 80 points
// (the 16-point rule on the triangle and on its four halves-of-edges
// subtriangles): okv / okp tell whether FP32 settles the kind-0 (v, three
// values) / kind-1 (p) integral, i.e. |coarse - refined| <= tol |coarse| / 2;
// v and p are then the refined values.
__device__ void dsm_first_level2_f32(double tol, const DsmTriF& T, float3 xc, float3 q, float3 R0, float3 R1,
                                     float3 R2, float area, double v[3], double p[1], bool& okv, bool& okp) {
    float coarse[4];
    dsm_rule2_f(T, xc, q, R0, R1, R2, area, coarse);
    const float3 m0 = fmid(R1, R2), m1 = fmid(R2, R0), m2 = fmid(R0, R1);
    const float sub = 0.25f * area;
    float a[4], b[4], c[4], d[4];
    dsm_rule2_f(T, xc, q, R0, m1, m2, sub, a);
    dsm_rule2_f(T, xc, q, m0, R1, m2, sub, b);
    dsm_rule2_f(T, xc, q, m0, m1, R2, sub, c);
    dsm_rule2_f(T, xc, q, m0, m1, m2, sub, d);
    // the sums and the test in FP32 (GB300's FP64 pipe runs at 1/64 of the FP32 rate): their rounding,
    // ~1e-7 of |coarse|, is far inside the factor-2 margin of the test (tol / 2 = 5e-4 of |coarse|)
    float ref[4], dnv = 0.f, cnv = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) ref[k] = (a[k] + b[k]) + (c[k] + d[k]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float e = coarse[k] - ref[k];
        dnv = fmaf(e, e, dnv);
        cnv = fmaf(coarse[k], coarse[k], cnv);
    }
    const float ht = 0.5f * (float)tol;
    okv = dnv <= ht * ht * cnv;
    okp = fabsf(coarse[3] - ref[3]) <= ht * fabsf(coarse[3]);
    for (int k = 0; k < 3; ++k) v[k] = ref[k];
    p[0] = ref[3];
}

// FP32 first-level record of a triangle (coordinates relative to its
// centroid, kept in FP64), built once per DipSourceMat launch.
struct DsmRecF {
    DsmTriF T;
    float3 F1, F2;   // vertices 1 and 2 relative to the centroid (vertex 0 is T.p0)
    float area;
    double cx, cy, cz;
};

__global__ void dsm_prepare_f_kernel(int64_t nt, const double* __restrict__ srec, DsmRecF* rec) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const double* s = srec + t * SREC;
    const d3 R0 = dev::ld3(s), R1 = dev::ld3(s + 3), R2 = dev::ld3(s + 6), n = dev::ld3(s + 9);
    const d3 e10 = R1 - R0, e20 = R2 - R0;
    const double c11 = dev::dot(e10, e10), c12 = dev::dot(e10, e20), c22 = dev::dot(e20, e20);
    const double inv_det = 1.0 / (c11 * c22 - c12 * c12);
    const d3 c = (R0 + R1 + R2) * (1.0 / 3.0);
    const d3 a0 = R0 - c, a1 = R1 - c, a2 = R2 - c;
    DsmRecF r;
    r.T.p0 = make_float3((float)a0.x, (float)a0.y, (float)a0.z);
    r.T.n = make_float3((float)n.x, (float)n.y, (float)n.z);
    r.T.e10 = make_float3((float)e10.x, (float)e10.y, (float)e10.z);
    r.T.e20 = make_float3((float)e20.x, (float)e20.y, (float)e20.z);
    r.T.d11 = (float)(c22 * inv_det);
    r.T.d12 = (float)(-c12 * inv_det);
    r.T.d22 = (float)(c11 * inv_det);
    r.F1 = make_float3((float)a1.x, (float)a1.y, (float)a1.z);
    r.F2 = make_float3((float)a2.x, (float)a2.y, (float)a2.z);
    r.area = (float)s[12];
    r.cx = c.x;
    r.cy = c.y;
    r.cz = c.z;
    rec[t] = r;
}

// Pair (dipole i, triangle t) of the DipSourceMat: the triangle's geometry
// for the integrator and the boundary coefficient, or false when the pair
// contributes nothing (dipole in no domain or a zero-conductivity one,
// triangle not on a boundary of the dipole's domain).
struct DsmPair {
    DsmTri T;
    d3 r0, q, R0, R1, R2;
    double area, coeffD, sigma;
    int m;
};

// The boundary coefficient of the pair, or false when it contributes nothing.
__device__ __forceinline__ bool dsm_pair_coeff(int64_t i, int64_t t, const int32_t* __restrict__ tmesh,
                                               const int* __restrict__ orient, const int* __restrict__ dom, int maxb,
                                               const int* __restrict__ dnb, const int* __restrict__ bmesh,
                                               const int* __restrict__ binside, const double* __restrict__ dsigma,
                                               DsmPair& P) {
    const int d = dom[i];
    if (d < 0) return false;
    P.sigma = dsigma[d];
    if (P.sigma == 0.0) return false;
    P.m = tmesh[t];
    bool on = false;
    for (int k = 0; k < dnb[d]; ++k)
        if (bmesh[d * maxb + k] == P.m) {
            P.coeffD = (binside[d * maxb + k] ? -kK : kK) * orient[d * maxb + k];
            on = true;
        }
    return on;
}

__device__ __forceinline__ bool dsm_pair(int64_t i, int64_t t, const double* __restrict__ dip,
                                         const double* __restrict__ srec, const int32_t* __restrict__ tmesh,
                                         const int* __restrict__ orient, const int* __restrict__ dom, int maxb,
                                         const int* __restrict__ dnb, const int* __restrict__ bmesh,
                                         const int* __restrict__ binside, const double* __restrict__ dsigma,
                                         DsmPair& P) {
    if (!dsm_pair_coeff(i, t, tmesh, orient, dom, maxb, dnb, bmesh, binside, dsigma, P)) return false;
    const double* s = srec + t * SREC;
    P.R0 = dev::ld3(s);
    P.R1 = dev::ld3(s + 3);
    P.R2 = dev::ld3(s + 6);
    P.T.p0 = P.R0;
    P.T.n = dev::ld3(s + 9);
    P.T.e10 = P.R1 - P.R0;
    P.T.e20 = P.R2 - P.R0;
    const double c11 = dev::dot(P.T.e10, P.T.e10), c12 = dev::dot(P.T.e10, P.T.e20),
                 c22 = dev::dot(P.T.e20, P.T.e20);
    const double inv_det = 1.0 / (c11 * c22 - c12 * c12);
    P.T.d11 = c22 * inv_det;
    P.T.d12 = -c12 * inv_det;
    P.T.d22 = c11 * inv_det;
    P.r0 = dev::ld3(dip + 6 * i);
    P.q = dev::ld3(dip + 6 * i + 3);
    P.area = s[12];
    return true;
}

// SourceMatrix<Dipole> (assembleSourceMat.cpp:66-104) with
// operatorPotentialDerivative / operatorPotential (operators.cpp:40-88):
// one thread per (dipole, triangle).  P0 rows are written directly (one
// triangle per row); the three P1 contributions go to `p1tmp` for a
// fixed-order vertex gather (the reference accumulates them atomically).
// Mixed precision: a pair whose first adaptive level FP32 settles is written
// here; the others are listed (with which of the two integrals is left) for
// the FP64 adaptive integration in dsm_fallback_kernel, so the warps of that
// deep recursion are not held up by pairs that need none.
constexpr int DSM_T_BITS = 29;   // triangle index bits of a list entry; the two top bits: integrals left

__global__ void dsm_kernel(int64_t dip0, int64_t ndc, const double* __restrict__ dip, int64_t nt,
                           const double* __restrict__ srec, const int32_t* __restrict__ tmesh,
                           const int64_t* __restrict__ tidx_ref, const int* __restrict__ barrier,
                           const int* __restrict__ orient, const int* __restrict__ dom, int maxb,
                           const int* __restrict__ dnb, const int* __restrict__ bmesh,
                           const int* __restrict__ binside, const double* __restrict__ dsigma, int order, int levels,
                           double tol, int64_t nv, int64_t nP, int perm, double* out, int64_t ldo, double* p1tmp,
                           int mixed, const DsmRecF* __restrict__ recf, int2* left, int* nleft) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t il = blockIdx.y;
    if (t >= nt || il >= ndc) return;
    const int64_t i = dip0 + il;
    double* o3 = p1tmp + (il * nt + t) * 3;
    o3[0] = o3[1] = o3[2] = 0.0;
    DsmPair P;
    const int64_t ref = tidx_ref[t];
    const int64_t row = perm ? ref - nv : ref;
    if (mixed && order == 3 && levels > 0) {
        if (!dsm_pair_coeff(i, t, tmesh, orient, dom, maxb, dnb, bmesh, binside, dsigma, P)) return;
        const bool p0row = !barrier[P.m];
        const DsmRecF R = recf[t];
        const double* dp = dip + 6 * i;
        const float3 xc = make_float3((float)(R.cx - dp[0]), (float)(R.cy - dp[1]), (float)(R.cz - dp[2]));
        const float3 qf = make_float3((float)dp[3], (float)dp[4], (float)dp[5]);
        double v[3], pf[1];
        bool f32v, f32p;
        dsm_first_level2_f32(tol, R.T, xc, qf, R.T.p0, R.F1, R.F2, R.area, v, pf, f32v, f32p);
        f32p = f32p && p0row;
        // FP32-accurate values: scaled in FP32 (an FP64 division per pair costs more than the pair's
        // FP32 work on GB300)
        const float cf = (float)P.coeffD;
        if (f32v) {
            o3[0] = (double)((float)v[0] * cf);
            o3[1] = (double)((float)v[1] * cf);
            o3[2] = (double)((float)v[2] * cf);
        }
        if (f32p) out[row + i * ldo] = (double)((float)pf[0] * (cf / (float)P.sigma));
        const int need = (f32v ? 0 : 1) | (p0row && !f32p ? 2 : 0);
        if (need) left[atomicAdd(nleft, 1)] = make_int2((int)il, (int)t | (need << DSM_T_BITS));
        return;
    }
    if (!dsm_pair(i, t, dip, srec, tmesh, orient, dom, maxb, dnb, bmesh, binside, dsigma, P)) return;
    const bool p0row = !barrier[P.m];
    double v[3];
    dsm_adaptive(0, order, levels, tol, P.T, P.r0, P.q, P.R0, P.R1, P.R2, P.area, v);
    o3[0] = v[0] * P.coeffD;
    o3[1] = v[1] * P.coeffD;
    o3[2] = v[2] * P.coeffD;
    if (p0row) {
        double p[3];
        dsm_adaptive(1, order, levels, tol, P.T, P.r0, P.q, P.R0, P.R1, P.R2, P.area, p);
        out[row + i * ldo] = p[0] * (P.coeffD / P.sigma);
    }
}

// The listed pairs of the mixed first pass: FP64 adaptive integration of the
// integrals FP32 did not settle (grid-stride over the device-side count, four
// lanes per pair; block size a multiple of 32).
__global__ void dsm_fallback_kernel(int64_t dip0, int64_t nt, const double* __restrict__ dip,
                                    const double* __restrict__ srec, const int32_t* __restrict__ tmesh,
                                    const int64_t* __restrict__ tidx_ref, const int* __restrict__ orient,
                                    const int* __restrict__ dom, int maxb, const int* __restrict__ dnb,
                                    const int* __restrict__ bmesh, const int* __restrict__ binside,
                                    const double* __restrict__ dsigma, int order, int levels, double tol, int64_t nv,
                                    int perm, double* out, int64_t ldo, double* p1tmp, const int2* __restrict__ left,
                                    const int* __restrict__ nleft) {
    // one group of four lanes per listed pair (the children of every node are integrated in parallel)
    const int n = *nleft;
    const int lane = threadIdx.x & 31, lane4 = lane & 3;
    const unsigned mask = 0xFu << (lane & ~3);
    const int groups = (int)(gridDim.x * blockDim.x / 4);
    for (int idx = (int)((blockIdx.x * blockDim.x + threadIdx.x) / 4); idx < n; idx += groups) {
        const int2 e = left[idx];
        const int64_t il = e.x, t = e.y & ((1 << DSM_T_BITS) - 1);
        const int need = (int)((unsigned)e.y >> DSM_T_BITS);
        const int64_t i = dip0 + il;
        DsmPair P;
        if (!dsm_pair(i, t, dip, srec, tmesh, orient, dom, maxb, dnb, bmesh, binside, dsigma, P)) continue;
        if (need & 1) {
            double v[3];
            dsm_adaptive_g4(0, order, levels, tol, P.T, P.r0, P.q, P.R0, P.R1, P.R2, P.area, v, mask, lane4);
            if (lane4 == 0) {
                double* o3 = p1tmp + (il * nt + t) * 3;
                o3[0] = v[0] * P.coeffD;
                o3[1] = v[1] * P.coeffD;
                o3[2] = v[2] * P.coeffD;
            }
        }
        if (need & 2) {
            double p[3];
            dsm_adaptive_g4(1, order, levels, tol, P.T, P.r0, P.q, P.R0, P.R1, P.R2, P.area, p, mask, lane4);
            const int64_t ref = tidx_ref[t];
            if (lane4 == 0) out[(perm ? ref - nv : ref) + i * ldo] = p[0] * (P.coeffD / P.sigma);
        }
    }
}

__global__ void dsm_gather_kernel(int64_t dip0, int64_t ndc, int64_t nv, int64_t nt, const double* __restrict__ p1tmp,
                                  const int32_t* __restrict__ v2t_beg, const int32_t* __restrict__ v2t_tri,
                                  const int8_t* __restrict__ v2t_loc, int64_t nP, int perm, double* out,
                                  int64_t ldo) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t il = blockIdx.y;
    if (v >= nv || il >= ndc) return;
    double sum = 0.0;
    bool any = false;
    for (int k = v2t_beg[v]; k < v2t_beg[v + 1]; ++k) {
        const double x = p1tmp[(il * nt + v2t_tri[k]) * 3 + v2t_loc[k]];
        if (x != 0.0) any = true;
        sum += x;
    }
    if (any) out[(perm ? nP + v : v) + (dip0 + il) * ldo] = sum;
}

// Danielsson's point-triangle distance (danielsson.cpp:26-74) with every
// operation rounded separately, in the reference's order (Vect3 dotprod and
// norm, vect3.h:72-73,111): no contraction into fused multiply-adds, so the
// distances equal the reference's double-precision ones bit for bit.  A point
// above an edge shared by two triangles is mathematically equidistant from
// both; which one is "nearest" is decided by the rounding of these
// operations, and EITSourceMat injects current into that triangle (and
// Head2EEGMat, with several interfaces, pairs it with another's weights).
__device__ __forceinline__ double dot_rn(d3 a, d3 b) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z));
}
__device__ __forceinline__ d3 sub_rn(d3 a, d3 b) {
    return {__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)};
}
__device__ double danielsson_rn(d3 p, const d3 P[3], double al[3]) {
    int idx[3] = {0, 1, 2};
    int nb = 3;
    al[0] = al[1] = al[2] = 0.0;
    for (;;) {
        if (nb == 1) {
            al[idx[0]] = 1.0;
            const d3 d = sub_rn(p, P[idx[0]]);
            return __dsqrt_rn(dot_rn(d, d));
        }
        d3 A0Ai[3];
        for (int i = 1; i < nb; ++i) A0Ai[i] = sub_rn(P[idx[i]], P[idx[0]]);
        const d3 A0M = sub_rn(p, P[idx[0]]);
        if (nb == 2) {
            al[idx[1]] = __ddiv_rn(dot_rn(A0M, A0Ai[1]), dot_rn(A0Ai[1], A0Ai[1]));
            al[idx[0]] = __dsub_rn(1.0, al[idx[1]]);
        } else {
            const double a00 = dot_rn(A0Ai[1], A0Ai[1]), a10 = dot_rn(A0Ai[1], A0Ai[2]),
                         a11 = dot_rn(A0Ai[2], A0Ai[2]);
            const double b0 = dot_rn(A0M, A0Ai[1]), b1 = dot_rn(A0M, A0Ai[2]);
            const double dd = __dsub_rn(__dmul_rn(a00, a11), __dmul_rn(a10, a10));
            al[idx[1]] = __ddiv_rn(__dsub_rn(__dmul_rn(b0, a11), __dmul_rn(b1, a10)), dd);
            al[idx[2]] = __ddiv_rn(__dsub_rn(__dmul_rn(a00, b1), __dmul_rn(a10, b0)), dd);
            al[idx[0]] = __dsub_rn(__dsub_rn(1.0, al[idx[1]]), al[idx[2]]);
        }
        int neg = -1;
        for (int i = 0; i < nb; ++i)
            if (al[idx[i]] < 0) {
                neg = i;
                break;
            }
        if (neg >= 0) {
            al[idx[neg]] = 0;
            const int tmp = idx[neg];
            idx[neg] = idx[nb - 1];
            idx[nb - 1] = tmp;
            --nb;
            continue;
        }
        d3 MH = {-A0M.x, -A0M.y, -A0M.z};
        for (int i = 1; i < nb; ++i) {
            const double a = al[idx[i]];
            MH = {__dadd_rn(MH.x, __dmul_rn(a, A0Ai[i].x)), __dadd_rn(MH.y, __dmul_rn(a, A0Ai[i].y)),
                  __dadd_rn(MH.z, __dmul_rn(a, A0Ai[i].z))};
        }
        return __dsqrt_rn(dot_rn(MH, MH));
    }
}

// ---- Head2EEGMat (assembleSensors.cpp:25-39): nearest triangle by Danielsson's
// point-triangle distance over the interfaces that touch a zero-conductivity
// domain (dist_point_geom, danielsson.cpp:107-128), one CTA per electrode, a
// fixed-order min reduction per interface (candidate segment).  The interfaces
// are visited in the reference's order and each one leaves the weights of its
// own nearest triangle in the shared result, so the electrode's weights are
// those of the last interface's nearest triangle while its triangle is the
// overall nearest (first strictly smaller distance) -- as the reference does.
__global__ void h2em_kernel(const double* __restrict__ pos, int nseg, const int64_t* __restrict__ seg,
                            const int32_t* __restrict__ cand, const double* __restrict__ srec,
                            const int32_t* __restrict__ T, const int64_t* __restrict__ vglob, int64_t nP, int perm,
                            double* dense, int64_t rs, int64_t cs, int64_t col0, int64_t* scols, double* svals) {
    __shared__ double sd[256];
    __shared__ int64_t so[256];
    __shared__ double sa[256][3];
    const int64_t e = blockIdx.x;
    const d3 p = dev::ld3(pos + 3 * e);
    double gbest = 1.79769313486231570e+308, w[3] = {0, 0, 0};
    int64_t gtri = -1;
    for (int q = 0; q < nseg; ++q) {
        double best = 1.79769313486231570e+308, bal[3] = {0, 0, 0};
        int64_t bo = INT64_MAX;
        for (int64_t k = seg[q] + threadIdx.x; k < seg[q + 1]; k += blockDim.x) {
            const double* s = srec + (int64_t)cand[k] * SREC;
            const d3 P[3] = {dev::ld3(s), dev::ld3(s + 3), dev::ld3(s + 6)};
            double al[3];
            const double dist = danielsson_rn(p, P, al);
            if (dist < best) {
                best = dist;
                bo = k;
                bal[0] = al[0]; bal[1] = al[1]; bal[2] = al[2];
            }
        }
        sd[threadIdx.x] = best;
        so[threadIdx.x] = bo;
        sa[threadIdx.x][0] = bal[0]; sa[threadIdx.x][1] = bal[1]; sa[threadIdx.x][2] = bal[2];
        __syncthreads();
        for (int wd = blockDim.x / 2; wd > 0; wd >>= 1) {
            if (threadIdx.x < wd) {
                const int o = threadIdx.x + wd;
                if (sd[o] < sd[threadIdx.x] || (sd[o] == sd[threadIdx.x] && so[o] < so[threadIdx.x])) {
                    sd[threadIdx.x] = sd[o];
                    so[threadIdx.x] = so[o];
                    sa[threadIdx.x][0] = sa[o][0]; sa[threadIdx.x][1] = sa[o][1]; sa[threadIdx.x][2] = sa[o][2];
                }
            }
            __syncthreads();
        }
        if (so[0] != INT64_MAX) {
            if (sd[0] < gbest) {
                gbest = sd[0];
                gtri = cand[so[0]];
            }
            w[0] = sa[0][0]; w[1] = sa[0][1]; w[2] = sa[0][2];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && gtri >= 0) {
        for (int j = 0; j < 3; ++j) {
            const int64_t v = vglob ? vglob[T[3 * gtri + j]] : T[3 * gtri + j];   // distinct vertex
            if (dense) dense[(perm ? nP + v : v) * rs + (col0 + e) * cs] = w[j];
            if (scols) scols[3 * e + j] = v;
            if (svals) svals[3 * e + j] = w[j];
        }
    }
}

// ---- Head2MEGMat (assembleSensors.cpp:69-96, assembleFerguson.cpp:18-31,
// operators.h:40-61): OperatorS of every triangle at every sensor, then a
// fixed-order gather per (sensor, vertex) of (B-A) S / (2 A).
__global__ void ferguson_s_kernel(const double* __restrict__ sq, int64_t np, int64_t nt,
                                  const double* __restrict__ srec, double* F) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    for (int64_t i = blockIdx.y; i < np; i += gridDim.y)
        F[i * nt + t] = dev::operator_S(srec + t * SREC, dev::ld3(sq + 6 * i));
}

__global__ void ferguson_gather_kernel(const double* __restrict__ sq, int64_t np, int64_t nv, int64_t nt,
                                       const double* __restrict__ F, const double* __restrict__ srec,
                                       const int32_t* __restrict__ v2t_beg, const int32_t* __restrict__ v2t_tri,
                                       const int8_t* __restrict__ v2t_loc, const int32_t* __restrict__ tmesh,
                                       const double* __restrict__ jump, int64_t nP, int perm, double* out,
                                       int64_t rs, int64_t cs, int64_t col0, double mag) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nv) return;
    for (int64_t i = blockIdx.y; i < np; i += gridDim.y) {
        d3 res = dev::mk(0, 0, 0);
        double coeff = 0.0;
        for (int k = v2t_beg[v]; k < v2t_beg[v + 1]; ++k) {
            const int64_t t = v2t_tri[k];
            const int loc = v2t_loc[k];
            const double* s = srec + t * SREC;
            const d3 A = dev::ld3(s + 3 * ((loc + 1) % 3)), B = dev::ld3(s + 3 * ((loc + 2) % 3));
            res = res + (B - A) * (F[i * nt + t] / (2 * s[12]));
            coeff = jump ? mag * jump[tmesh[t]] : mag;
        }
        const d3 o = dev::ld3(sq + 6 * i + 3);
        out[(perm ? nP + v : v) * rs + (col0 + i) * cs] = dev::dot(res * coeff, o) / dev::norm(o);
    }
}

// ---- DipSource2MEGMat (assembleSensors.cpp:133-159): Biot-Savart primary field.
__global__ void ds2mm_kernel(const double* __restrict__ dip, int64_t nd, const double* __restrict__ sq, int64_t np,
                             double* out, int64_t ldo) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= np) return;
    const d3 o = dev::ld3(sq + 6 * i + 3);
    for (int64_t j = blockIdx.y; j < nd; j += gridDim.y) {
        const d3 r = dev::ld3(dip + 6 * j), q = dev::ld3(dip + 6 * j + 3);
        const d3 diff = dev::ld3(sq + 6 * i) - r;
        const double nd3 = dev::norm(diff);
        const d3 f = dev::cross(q, diff) * (1.0 / (nd3 * nd3 * nd3));
        out[i + j * ldo] = dev::dot(f, o) * kMagFactor / dev::norm(o);
    }
}

void launch_mesh_solid_angles(const double* pts, int64_t pstride, int64_t n, int nmesh, const int64_t* tbeg_dev,
                              const double* srec, double* out, cudaStream_t s, bool screened) {
    if (n == 0) return;
    ProfScope prof_("solid_angles", s);
    if (screened)
        mesh_solid_angles_screened_kernel<<<(unsigned)n, 256, 0, s>>>(pts, pstride, nmesh, tbeg_dev, srec, out);
    else
        mesh_solid_angles_kernel<<<(unsigned)n, 256, 0, s>>>(pts, pstride, nmesh, tbeg_dev, srec, out);
    check_launch("mesh solid angles");
}

void launch_domain_lookup(int64_t n, int nmesh, const double* sa, int ndom, int maxb, const int* dnb,
                          const int* bmesh, const int* binside, const int* borient, const int* bgrp, int forced,
                          int* dom, int* err, cudaStream_t s) {
    ProfScope prof_("domain_lookup", s);
    if (n == 0) return;
    domain_lookup_kernel<<<nblocks(n, 128), 128, 0, s>>>(n, nmesh, sa, ndom, maxb, dnb, bmesh, binside, borient,
                                                         bgrp, forced, dom, err);
    check_launch("domain lookup");
}

// Dipoles whose domain lies outside a planned set (bit d of `allowed`): the
// row ranges of a planned gain contraction would miss their DipSourceMat rows.
// Flags OMG_ERR_INVALID with err[1] = 1 and the first such dipole in err[2].
__global__ void domain_check_kernel(int64_t n, const int* __restrict__ dom, uint64_t allowed, int* err) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int d = dom[i];
    if (d < 0 || (d < 64 && ((allowed >> d) & 1ull))) return;   // d < 0 is flagged by the lookup itself
    if (atomicCAS(err, 0, OMG_ERR_INVALID) == 0) {
        err[1] = 1;
        err[2] = (int)i;
    }
}

void launch_domain_check(int64_t n, const int* dom, uint64_t allowed, int* err, cudaStream_t s) {
    if (n == 0) return;
    domain_check_kernel<<<nblocks(n, 128), 128, 0, s>>>(n, dom, allowed, err);
    check_launch("domain check");
}

void launch_dsm(const DevGeom& g, int64_t dip0, int64_t ndc, const double* dip, const int32_t* tmesh,
                const int64_t* tidx_ref, const int* barrier, const int* orient, const int* dom, int maxb,
                const int* dnb, const int* bmesh, const int* binside, const double* dsigma, int order, int levels,
                double tol, int perm, double* out, int64_t ldo, double* p1tmp, int mixed, cudaStream_t s) {
    ProfScope prof_("dsm", s);
    if (ndc == 0) return;
    if (g.nt >= ((int64_t)1 << DSM_T_BITS) || ndc > INT32_MAX) throw Error(OMG_ERR_UNSUPPORTED, "DSM: too many triangles");
    const bool two_pass = mixed && order == 3 && levels > 0;
    // the pairs FP32 does not settle (at most one entry per pair) and their count
    DevBuf left(two_pass ? (size_t)ndc * g.nt * sizeof(int2) : 0, s), nleft(two_pass ? sizeof(int) : 0, s),
        recf(two_pass ? (size_t)g.nt * sizeof(DsmRecF) : 0, s);
    if (two_pass) {
        OMG_CUDA(cudaMemsetAsync(nleft.p, 0, sizeof(int), s));
        dsm_prepare_f_kernel<<<nblocks(g.nt, 128), 128, 0, s>>>(g.nt, g.srec, static_cast<DsmRecF*>(recf.p));
        check_launch("DSM records");
    }
    dim3 grid(nblocks(g.nt, 128), (unsigned)ndc);
    dsm_kernel<<<grid, 128, 0, s>>>(dip0, ndc, dip, g.nt, g.srec, tmesh, tidx_ref, barrier, orient, dom, maxb, dnb,
                                    bmesh, binside, dsigma, order, levels, tol, g.nvg, g.nP, perm, out, ldo, p1tmp, mixed,
                                    static_cast<const DsmRecF*>(recf.p), left.as<int2>(), nleft.as<int>());
    check_launch("DSM");
    if (two_pass) {
        static int n_sm = 0;
        if (!n_sm) {
            int dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
            if (n_sm <= 0) n_sm = 1;
        }
        dsm_fallback_kernel<<<(unsigned)(n_sm * 8), 128, 0, s>>>(dip0, g.nt, dip, g.srec, tmesh, tidx_ref, orient, dom,
                                                                  maxb, dnb, bmesh, binside, dsigma, order, levels,
                                                                  tol, g.nvg, perm, out, ldo, p1tmp, left.as<int2>(),
                                                                  nleft.as<int>());
        check_launch("DSM (FP64 pairs)");
    }
    dim3 grid2(nblocks(g.nv, 128), (unsigned)ndc);
    dsm_gather_kernel<<<grid2, 128, 0, s>>>(dip0, ndc, g.nv, g.nt, p1tmp, g.v2t_beg, g.v2t_tri, g.v2t_loc, g.nP,
                                            perm, out, ldo);
    check_launch("DSM gather");
}

void launch_h2em(const DevGeom& g, const double* pos, int64_t ne, int nseg, const int64_t* seg, const int32_t* cand,
                 int perm, double* dense, int64_t rs, int64_t cs, int64_t col0, int64_t* scols, double* svals,
                 cudaStream_t s) {
    if (ne == 0) return;
    ProfScope prof_("h2em", s);
    h2em_kernel<<<(unsigned)ne, 256, 0, s>>>(pos, nseg, seg, cand, g.srec, g.T, g.vglob, g.nP, perm, dense, rs, cs,
                                             col0, scols, svals);
    check_launch("H2EM");
}

void launch_h2mm(const DevGeom& g, const double* sq, int64_t np, const int32_t* tmesh, const double* jump, int perm,
                 double* out, int64_t rs, int64_t cs, int64_t col0, double* F, cudaStream_t s, double mag) {
    ProfScope prof_("h2mm", s);
    if (np == 0) return;
    dim3 grid(nblocks(g.nt, 128), (unsigned)std::min<int64_t>(np, 32768));
    ferguson_s_kernel<<<grid, 128, 0, s>>>(sq, np, g.nt, g.srec, F);
    check_launch("Ferguson S");
    dim3 grid2(nblocks(g.nv, 128), (unsigned)std::min<int64_t>(np, 32768));
    ferguson_gather_kernel<<<grid2, 128, 0, s>>>(sq, np, g.nv, g.nt, F, g.srec, g.v2t_beg, g.v2t_tri, g.v2t_loc,
                                                 tmesh, jump, g.nP, perm, out, rs, cs, col0, mag);
    check_launch("Ferguson gather");
}

void launch_ds2mm(const double* dip, int64_t nd, const double* sq, int64_t np, double* out, int64_t ldo,
                  cudaStream_t s) {
    ProfScope prof_("ds2mm", s);
    if (nd == 0 || np == 0) return;
    dim3 grid(nblocks(np, 128), (unsigned)std::min<int64_t>(nd, 32768));
    ds2mm_kernel<<<grid, 128, 0, s>>>(dip, nd, sq, np, out, ldo);
    check_launch("DS2MM");
}

// ===========================================================================
// DipSourceMat vector-Jacobian product: for each dipole j,
//   d/d(r0_j, q_j) of  sum_rows U[row, j] * DSM[row, j]
// from the analytic derivatives of the integrands (Dipole::potential and
// Dipole::gradient, dipole.h:29-46) integrated over the same adaptive trees as
// the forward assembly (integrator.h:228-252): refinement decisions come from
// the forward integrand, so this is the exact derivative of the assembled
// (piecewise) DSM.
// ===========================================================================
struct VjpW {
    double W[3];   // U at the triangle's vertices x coeffD (P1 rows)
    double w0;     // U at the triangle's row x coeffD / sigma (P0 row; 0 on current barriers)
};

// Derivative integrand: kind 0 -> w1(r) * d g / d(r0, q); kind 1 -> w0 * d p / d(r0, q).
__device__ __forceinline__ void dsm_vjp_point(int kind, const DsmTri& T, d3 r0, d3 q, d3 r, const VjpW& w,
                                              double out[6]) {
    const d3 x = r - r0;
    const double inv = 1.0 / dev::dot(x, x);
    const double inv3 = inv * sqrt(inv), inv5 = inv3 * inv, inv7 = inv5 * inv;
    const double qx = dev::dot(q, x);
    if (kind == 1) {
        // p = (q.x)/|x|^3 ; dp/dq = x/|x|^3 ; dp/dr0 = -(q/|x|^3 - 3 (q.x) x/|x|^5)
        const d3 dq = x * inv3;
        const d3 dx = q * inv3 - x * (3.0 * qx * inv5);
        out[0] = -w.w0 * dx.x; out[1] = -w.w0 * dx.y; out[2] = -w.w0 * dx.z;
        out[3] = w.w0 * dq.x; out[4] = w.w0 * dq.y; out[5] = w.w0 * dq.z;
        return;
    }
    const d3 n = T.n;
    const double xn = dev::dot(x, n), qn = dev::dot(q, n);
    // g = (q.n)/|x|^3 - 3 (q.x)(x.n)/|x|^5
    const d3 dq = n * inv3 - x * (3.0 * xn * inv5);
    const d3 dx = x * (-3.0 * qn * inv5 + 15.0 * qx * xn * inv7) - q * (3.0 * xn * inv5) - n * (3.0 * qx * inv5);
    const d3 v = r - T.p0;
    const double a1 = dev::dot(v, T.e10), a2 = dev::dot(v, T.e20);
    const double l1 = T.d11 * a1 + T.d12 * a2, l2 = T.d12 * a1 + T.d22 * a2, l0 = 1.0 - l1 - l2;
    const double w1 = w.W[0] * l0 + w.W[1] * l1 + w.W[2] * l2;
    out[0] = -w1 * dx.x; out[1] = -w1 * dx.y; out[2] = -w1 * dx.z;
    out[3] = w1 * dq.x; out[4] = w1 * dq.y; out[5] = w1 * dq.z;
}

__device__ __forceinline__ void dsm_vjp_rule(int kind, int order, const DsmTri& T, d3 r0, d3 q, const VjpW& w,
                                             d3 P0, d3 P1, d3 P2, double area, double acc[6]) {
    double s[6] = {0, 0, 0, 0, 0, 0};
    const int np = c_nbpts[order];
    for (int k = 0; k < np; ++k) {
        const d3 xk = bary_point(c_rules[order][k], P0, P1, P2);
        double e[6];
        dsm_vjp_point(kind, T, r0, q, xk, w, e);
        const double wk = c_rules[order][k][3];
        for (int c = 0; c < 6; ++c) s[c] += wk * e[c];
    }
    for (int c = 0; c < 6; ++c) acc[c] += area * s[c];
}

// Same traversal as dsm_adaptive; accepted nodes contribute the derivative
// rule over their four children (the values the forward sums).
__device__ void dsm_vjp_adaptive(int kind, int order, int levels, double tol, const DsmTri& T, d3 r0, d3 q,
                                 const VjpW& w, d3 R0, d3 R1, d3 R2, double area, double grad[6]) {
    if (levels == 0) {
        dsm_vjp_rule(kind, order, T, r0, q, w, R0, R1, R2, area, grad);
        return;
    }
    double coarse[3];
    dsm_rule(kind, order, T, r0, q, R0, R1, R2, area, coarse);
    uint32_t st_path[DSM_STACK];
    int8_t st_depth[DSM_STACK], st_level[DSM_STACK];
    double st_c[DSM_STACK][3];
    int sp = 1;
    st_path[0] = 0; st_depth[0] = 0; st_level[0] = (int8_t)levels;
    st_c[0][0] = coarse[0]; st_c[0][1] = coarse[1]; st_c[0][2] = coarse[2];
    const int dim = kind == 0 ? 3 : 1;
    while (sp > 0) {
        --sp;
        const uint32_t path = st_path[sp];
        const int depth = st_depth[sp], level = st_level[sp];
        const double c0 = st_c[sp][0], c1 = st_c[sp][1], c2 = st_c[sp][2];
        d3 P0 = R0, P1 = R1, P2 = R2;
        double a = area;
        for (int d = 0; d < depth; ++d) {
            subtriangle(P0, P1, P2, (path >> (2 * d)) & 3);
            a *= 0.25;
        }
        const double sub = 0.25 * a;
        double integ[4][3];
        double ref[3] = {0.0, 0.0, 0.0};
        for (int c = 0; c < 4; ++c) {
            d3 Q0 = P0, Q1 = P1, Q2 = P2;
            subtriangle(Q0, Q1, Q2, c);
            dsm_rule(kind, order, T, r0, q, Q0, Q1, Q2, sub, integ[c]);
            for (int k = 0; k < dim; ++k) ref[k] += integ[c][k];
        }
        double dn, cn;
        if (dim == 1) {
            dn = fabs(c0 - ref[0]);
            cn = fabs(c0);
        } else {
            const double e0 = c0 - ref[0], e1 = c1 - ref[1], e2 = c2 - ref[2];
            dn = sqrt(e0 * e0 + e1 * e1 + e2 * e2);
            cn = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
        }
        if (dn <= tol * cn || level == 0) {
            for (int c = 0; c < 4; ++c) {
                d3 Q0 = P0, Q1 = P1, Q2 = P2;
                subtriangle(Q0, Q1, Q2, c);
                dsm_vjp_rule(kind, order, T, r0, q, w, Q0, Q1, Q2, sub, grad);
            }
            continue;
        }
        for (int c = 3; c >= 0; --c) {
            st_path[sp] = path | ((uint32_t)c << (2 * depth));
            st_depth[sp] = (int8_t)(depth + 1);
            st_level[sp] = (int8_t)(level - 1);
            st_c[sp][0] = integ[c][0]; st_c[sp][1] = integ[c][1]; st_c[sp][2] = integ[c][2];
            ++sp;
        }
    }
}

__global__ void dsm_vjp_kernel(int64_t dip0, int64_t ndc, const double* __restrict__ dip, int64_t nt,
                               const double* __restrict__ srec, const int32_t* __restrict__ T32,
                               const int32_t* __restrict__ tmesh, const int64_t* __restrict__ tidx_ref,
                               const int* __restrict__ barrier, const int* __restrict__ orient,
                               const int* __restrict__ dom, int maxb, const int* __restrict__ dnb,
                               const int* __restrict__ bmesh, const int* __restrict__ binside,
                               const double* __restrict__ dsigma, int order, int levels, double tol,
                               const double* __restrict__ U, int64_t ldu, double* part) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t il = blockIdx.y;
    if (t >= nt || il >= ndc) return;
    const int64_t i = dip0 + il;
    double* o = part + (il * nt + t) * 6;
    for (int c = 0; c < 6; ++c) o[c] = 0.0;
    const int d = dom[i];
    if (d < 0) return;
    const double sigma = dsigma[d];
    if (sigma == 0.0) return;
    const int m = tmesh[t];
    double coeffD = 0.0;
    bool on = false;
    for (int k = 0; k < dnb[d]; ++k)
        if (bmesh[d * maxb + k] == m) {
            coeffD = (binside[d * maxb + k] ? -kK : kK) * orient[d * maxb + k];
            on = true;
        }
    if (!on) return;
    const double* s = srec + t * SREC;
    const d3 R0 = dev::ld3(s), R1 = dev::ld3(s + 3), R2 = dev::ld3(s + 6);
    DsmTri T;
    T.p0 = R0;
    T.n = dev::ld3(s + 9);
    T.e10 = R1 - R0;
    T.e20 = R2 - R0;
    const double c11 = dev::dot(T.e10, T.e10), c12 = dev::dot(T.e10, T.e20), c22 = dev::dot(T.e20, T.e20);
    const double inv_det = 1.0 / (c11 * c22 - c12 * c12);
    T.d11 = c22 * inv_det;
    T.d12 = -c12 * inv_det;
    T.d22 = c11 * inv_det;
    const d3 r0 = dev::ld3(dip + 6 * i), q = dev::ld3(dip + 6 * i + 3);
    const double* Uj = U + i * ldu;
    VjpW w;
    for (int k = 0; k < 3; ++k) w.W[k] = Uj[T32[3 * t + k]] * coeffD;
    w.w0 = barrier[m] ? 0.0 : Uj[tidx_ref[t]] * (coeffD / sigma);
    double g[6] = {0, 0, 0, 0, 0, 0};
    dsm_vjp_adaptive(0, order, levels, tol, T, r0, q, w, R0, R1, R2, s[12], g);
    if (!barrier[m]) dsm_vjp_adaptive(1, order, levels, tol, T, r0, q, w, R0, R1, R2, s[12], g);
    for (int c = 0; c < 6; ++c) o[c] = g[c];
}

// Fixed-order sum over triangles: one CTA per dipole.
__global__ void dsm_vjp_reduce_kernel(int64_t dip0, int64_t ndc, int64_t nt, const double* __restrict__ part,
                                      double* out) {
    __shared__ double red[6][128];
    const int64_t il = blockIdx.x;
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t t = threadIdx.x; t < nt; t += 128)
        for (int c = 0; c < 6; ++c) acc[c] += part[(il * nt + t) * 6 + c];
    for (int c = 0; c < 6; ++c) red[c][threadIdx.x] = acc[c];
    __syncthreads();
    for (int w = 64; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int c = 0; c < 6; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 6) out[(dip0 + il) * 6 + threadIdx.x] = red[threadIdx.x][0];
}

void launch_dsm_vjp(const DevGeom& g, int64_t dip0, int64_t ndc, const double* dip, const int32_t* tmesh,
                    const int64_t* tidx_ref, const int* barrier, const int* orient, const int* dom, int maxb,
                    const int* dnb, const int* bmesh, const int* binside, const double* dsigma, int order, int levels,
                    double tol, const double* U, int64_t ldu, double* part, double* out, cudaStream_t s) {
    if (ndc == 0) return;
    ProfScope prof_("dsm_vjp", s);
    dim3 grid(nblocks(g.nt, 128), (unsigned)ndc);
    dsm_vjp_kernel<<<grid, 128, 0, s>>>(dip0, ndc, dip, g.nt, g.srec, g.T, tmesh, tidx_ref, barrier, orient, dom, maxb,
                                        dnb, bmesh, binside, dsigma, order, levels, tol, U, ldu, part);
    check_launch("DSM vjp");
    dsm_vjp_reduce_kernel<<<(unsigned)ndc, 128, 0, s>>>(dip0, ndc, g.nt, part, out);
    check_launch("DSM vjp reduce");
}

// ---------------------------------------------------------------------------
// Internal potentials.  Surf2VolMat (assembleHeadMat.cpp:325-363) through
// PartialBlock (operators.h:302-331): for a point x in a conducting domain and
// every mesh m bounding that domain, with c = K * mesh_orientation(domain, m)
// (domain.h:43-45),
//   row(x), vertex columns   += -c * P1SingleLayerPotential(triangle)(x)[k]
//   row(x), triangle column   =  c / sigma * OperatorS(triangle)(x)   (no current barrier)
// One thread per (triangle, point): the three P1 integrals go to a per-point
// scratch row (zero where the triangle's mesh does not bound the point's
// domain) and the S value straight to its column; a second pass sums the
// scratch over each vertex's triangles in triangle order, as the reference's
// loop accumulates them.  Rows are the kept points (rows[i] >= 0).
// ---------------------------------------------------------------------------
__global__ void partial_block_kernel(int64_t p0, int64_t npc, const double* __restrict__ pts,
                                     const int* __restrict__ pdom, const int64_t* __restrict__ rows, int64_t nt,
                                     const double* __restrict__ srec, const double* __restrict__ prec,
                                     const int32_t* __restrict__ tmesh, const int64_t* __restrict__ tidx_ref,
                                     const int* __restrict__ barrier, const int* __restrict__ orient, int maxb,
                                     const int* __restrict__ dnb, const int* __restrict__ bmesh,
                                     const int* __restrict__ binside, const double* __restrict__ dsigma,
                                     double* __restrict__ p1tmp, double* out, int64_t ldo, int64_t tshift) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t il = blockIdx.y;
    if (t >= nt || il >= npc) return;
    const int64_t i = p0 + il;
    double* o3 = p1tmp + (il * nt + t) * 3;
    o3[0] = o3[1] = o3[2] = 0.0;
    const int64_t row = rows[i];
    if (row < 0) return;
    const int d = pdom[i];
    const int m = tmesh[t];
    double c = 0.0;
    bool on = false;
    for (int k = 0; k < dnb[d]; ++k)
        if (bmesh[d * maxb + k] == m) {
            c = (binside[d * maxb + k] ? kK : -kK) * orient[d * maxb + k];
            on = true;
        }
    if (!on) return;
    const d3 x = dev::ld3(pts + 3 * i);
    double v[3];
    dev::p1_single_layer(prec + t * PREC, x, v);
    o3[0] = v[0] * -c;
    o3[1] = v[1] * -c;
    o3[2] = v[2] * -c;
    if (!barrier[m]) out[row + (tidx_ref[t] + tshift) * ldo] = (c / dsigma[d]) * dev::operator_S(srec + t * SREC, x);
}

__global__ void partial_block_gather_kernel(int64_t p0, int64_t npc, const int64_t* __restrict__ rows, int64_t nv,
                                            int64_t nt, const double* __restrict__ p1tmp,
                                            const int32_t* __restrict__ v2t_beg, const int32_t* __restrict__ v2t_tri,
                                            const int8_t* __restrict__ v2t_loc, double* out, int64_t ldo) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t il = blockIdx.y;
    if (v >= nv || il >= npc) return;
    const int64_t row = rows[p0 + il];
    if (row < 0) return;
    double sum = 0.0;
    for (int k = v2t_beg[v]; k < v2t_beg[v + 1]; ++k) sum += p1tmp[(il * nt + v2t_tri[k]) * 3 + v2t_loc[k]];
    out[row + v * ldo] = sum;
}

void launch_partial_block(const DevGeom& g, int64_t p0, int64_t npc, const double* pts, const int* pdom,
                          const int64_t* rows, const int32_t* tmesh, const int64_t* tidx_ref, const int* barrier,
                          const int* orient, int maxb, const int* dnb, const int* bmesh, const int* binside,
                          const double* dsigma, double* p1tmp, double* out, int64_t ldo, cudaStream_t s,
                          int64_t tshift) {
    if (npc == 0) return;
    ProfScope prof_("partial_block", s);
    dim3 grid(nblocks(g.nt, 128), (unsigned)npc);
    partial_block_kernel<<<grid, 128, 0, s>>>(p0, npc, pts, pdom, rows, g.nt, g.srec, g.prec, tmesh, tidx_ref,
                                              barrier, orient, maxb, dnb, bmesh, binside, dsigma, p1tmp, out, ldo,
                                              tshift);
    check_launch("partial block");
    dim3 grid2(nblocks(g.nv, 128), (unsigned)npc);
    partial_block_gather_kernel<<<grid2, 128, 0, s>>>(p0, npc, rows, g.nv, g.nt, p1tmp, g.v2t_beg, g.v2t_tri,
                                                      g.v2t_loc, out, ldo);
    check_launch("partial block gather");
}

// DipSource2InternalPotMat (assembleSourceMat.cpp:154-187): the infinite-medium
// potential K / sigma * q.(x - r0) / |x - r0|^3 (dipole.h:29-36) of each
// dipole at each kept point that shares its domain, zero elsewhere.
__global__ void dipole_internal_pot_kernel(const double* __restrict__ pts, const int* __restrict__ pdom,
                                           const int64_t* __restrict__ rows, int64_t np,
                                           const double* __restrict__ dip, const int* __restrict__ ddom, int64_t nd,
                                           const double* __restrict__ dsigma, double* out, int64_t ldo) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= np) return;
    const int64_t row = rows[i];
    if (row < 0) return;
    const int d = pdom[i];
    const d3 x = dev::ld3(pts + 3 * i);
    for (int64_t j = blockIdx.y; j < nd; j += gridDim.y) {
        double val = 0.0;
        if (ddom[j] == d) {
            const d3 r = x - dev::ld3(dip + 6 * j);
            const double n2 = dev::dot(r, r);
            val = (kK / dsigma[d]) * (dev::dot(dev::ld3(dip + 6 * j + 3), r) / (n2 * sqrt(n2)));
        }
        out[row + j * ldo] = val;
    }
}

void launch_dipole_internal_pot(const double* pts, const int* pdom, const int64_t* rows, int64_t np, const double* dip,
                                const int* ddom, int64_t nd, const double* dsigma, double* out, int64_t ldo,
                                cudaStream_t s) {
    if (np == 0 || nd == 0) return;
    ProfScope prof_("dipole_internal_pot", s);
    dim3 grid(nblocks(np, 128), (unsigned)std::min<int64_t>(nd, 32768));
    dipole_internal_pot_kernel<<<grid, 128, 0, s>>>(pts, pdom, rows, np, dip, ddom, nd, dsigma, out, ldo);
    check_launch("dipole internal potential");
}

// ---------------------------------------------------------------------------
// EITSourceMat (assembleSourceMat.cpp:109-152).  The reference fills the
// rows of a transfer matrix for the triangles of current-barrier meshes,
//   D(K o) over (injection triangle, vertices of mesh2)          (operators.h:83-115, 439-442)
//   -1/2 Id on the self pair, Id(t, v) = area / 3                (operators.h:200-206, 267-269)
//   S(-K o sigma_inv) over (injection triangle, triangles of mesh2 != mesh1)   (operators.h:391-425)
// and sums the rows of each electrode's injection triangles with its weight.
// Only the rows of injection triangles are computed here: R is row-major,
// one row of Nref (reference-numbered) columns per injection triangle.
// ---------------------------------------------------------------------------

// Nearest candidate triangle per electrode (dist_point_geom,
// danielsson.cpp:107-128): one CTA per electrode, ties to the first candidate
// (the reference keeps the first strictly smaller distance).
__global__ void nearest_triangle_kernel(const double* __restrict__ pos, int64_t ncand,
                                        const int32_t* __restrict__ cand, const double* __restrict__ srec,
                                        int64_t* out_tri) {
    __shared__ double sd[256];
    __shared__ int64_t so[256];
    const int64_t e = blockIdx.x;
    const d3 p = dev::ld3(pos + 3 * e);
    double best = 1.79769313486231570e+308;
    int64_t bo = INT64_MAX;
    for (int64_t k = threadIdx.x; k < ncand; k += blockDim.x) {
        const double* s = srec + (int64_t)cand[k] * SREC;
        const d3 P[3] = {dev::ld3(s), dev::ld3(s + 3), dev::ld3(s + 6)};
        double al[3];
        const double dist = danielsson_rn(p, P, al);
        if (dist < best) {
            best = dist;
            bo = k;
        }
    }
    sd[threadIdx.x] = best;
    so[threadIdx.x] = bo;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            const int o = threadIdx.x + w;
            if (sd[o] < sd[threadIdx.x] || (sd[o] == sd[threadIdx.x] && so[o] < so[threadIdx.x])) {
                sd[threadIdx.x] = sd[o];
                so[threadIdx.x] = so[o];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out_tri[e] = so[0] < ncand ? (int64_t)cand[so[0]] : -1;
}

void launch_nearest_triangle(const DevGeom& g, const double* pos, int64_t ne, int64_t ncand, const int32_t* cand,
                             int64_t* out_tri, cudaStream_t s) {
    if (ne == 0) return;
    ProfScope prof_("nearest_triangle", s);
    nearest_triangle_kernel<<<(unsigned)ne, 256, 0, s>>>(pos, ncand, cand, g.srec, out_tri);
    check_launch("nearest triangle");
}

// tmp[(k nb + j) 3 + l] = integral over injection triangle inj[k] of
// P1SingleLayerPotential(t2b + j), component l (the D block's pair integral).
__global__ void eit_d_kernel(const int64_t* __restrict__ inj, int64_t nk, const double* __restrict__ qrec,
                             const double* __restrict__ prec, int64_t t2b, int64_t nb, int order, double* tmp) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t k = blockIdx.y;
    if (j >= nb || k >= nk) return;
    const double* q = qrec + inj[k] * QREC;
    const double* P = prec + (t2b + j) * PREC;
    const int np = c_nbpts[order];
    double acc[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < np; ++i) {
        double v[3];
        dev::p1_single_layer(P, dev::ld3(q + 3 * i), v);
        const double w = c_rules[order][i][3];
        acc[0] += w * v[0];
        acc[1] += w * v[1];
        acc[2] += w * v[2];
    }
    double* o = tmp + (k * nb + j) * 3;
    o[0] = q[48] * acc[0];
    o[1] = q[48] * acc[1];
    o[2] = q[48] * acc[2];
}

// R[k, v] += coeffD * sum over the triangles of [t2b, t2b + nb) holding v (triangle order),
// then the -1/2 Id term of the self pair.
__global__ void eit_d_gather_kernel(const int64_t* __restrict__ inj, int64_t nk, int64_t t2b, int64_t nb, int64_t vb,
                                    int64_t nvb, double coeffD, int self, const double* __restrict__ tmp,
                                    const int32_t* __restrict__ v2t_beg, const int32_t* __restrict__ v2t_tri,
                                    const int8_t* __restrict__ v2t_loc, const int32_t* __restrict__ T,
                                    const double* __restrict__ srec, const int64_t* __restrict__ vglob, double* R,
                                    int64_t Nref) {
    const int64_t iv = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t k = blockIdx.y;
    if (iv >= nvb || k >= nk) return;
    const int64_t v = vb + iv;
    // the column of the vertex: a copy of a vertex shared by several meshes adds into its distinct vertex
    // (the copies are in different meshes, so different launches, one after the other)
    const int64_t col = vglob ? vglob[v] : v;
    double sum = 0.0;
    for (int q = v2t_beg[v]; q < v2t_beg[v + 1]; ++q) {
        const int64_t t2 = v2t_tri[q];
        if (t2 < t2b || t2 >= t2b + nb) continue;
        sum += tmp[(k * nb + (t2 - t2b)) * 3 + v2t_loc[q]];
    }
    double r = R[k * Nref + col] + coeffD * sum;
    if (self) {
        const int64_t u = inj[k];
        if (T[3 * u] == v || T[3 * u + 1] == v || T[3 * u + 2] == v) r += -0.5 * (srec[u * SREC + 12] / 3.0);
    }
    R[k * Nref + col] = r;
}

// R[k, tidx(t2)] = coeffS * integral over t2 of OperatorS(inj[k]).
__global__ void eit_s_kernel(const int64_t* __restrict__ inj, int64_t nk, const double* __restrict__ srec,
                             const double* __restrict__ qrec, int64_t t2b, int64_t nb, int order,
                             const int64_t* __restrict__ tidx_ref, double coeffS, double* R, int64_t Nref) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t k = blockIdx.y;
    if (j >= nb || k >= nk) return;
    const double* sr = srec + inj[k] * SREC;
    const double* q = qrec + (t2b + j) * QREC;
    const int np = c_nbpts[order];
    double acc = 0.0;
    for (int i = 0; i < np; ++i) acc += c_rules[order][i][3] * dev::operator_S(sr, dev::ld3(q + 3 * i));
    R[k * Nref + tidx_ref[t2b + j]] = (q[48] * acc) * coeffS;
}

void launch_eit_rows(const DevGeom& g, const int64_t* inj, int64_t nk, int64_t t2b, int64_t t2e, int64_t vb,
                     int64_t ve, bool self, bool withS, double coeffD, double coeffS, const int64_t* tidx_ref,
                     int order, double* tmp, double* R, cudaStream_t s) {
    if (nk == 0) return;
    ProfScope prof_("eit_rows", s);
    const int64_t nb = t2e - t2b;
    dim3 grid(nblocks(nb, 128), (unsigned)nk);
    eit_d_kernel<<<grid, 128, 0, s>>>(inj, nk, g.qrec, g.prec, t2b, nb, order, tmp);
    check_launch("EIT D");
    dim3 grid2(nblocks(ve - vb, 128), (unsigned)nk);
    eit_d_gather_kernel<<<grid2, 128, 0, s>>>(inj, nk, t2b, nb, vb, ve - vb, coeffD, self ? 1 : 0, tmp, g.v2t_beg,
                                              g.v2t_tri, g.v2t_loc, g.T, g.srec, g.vglob, R, g.Nref);
    check_launch("EIT D gather");
    if (withS) {
        eit_s_kernel<<<grid, 128, 0, s>>>(inj, nk, g.srec, g.qrec, t2b, nb, order, tidx_ref, coeffS, R, g.Nref);
        check_launch("EIT S");
    }
}

// out[i, e] += sum over the electrode's injection entries q with k0 <= id[q] < k0 + nk
// of coef[q] * R[id[q] - k0, i], in the electrode's triangle order.
__global__ void eit_combine_kernel(int64_t Nref, int64_t ne, const int64_t* __restrict__ ebeg,
                                   const int64_t* __restrict__ eid, const double* __restrict__ ecoef, int64_t k0,
                                   int64_t nk, const double* __restrict__ R, double* out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= Nref) return;
    for (int64_t e = blockIdx.y; e < ne; e += gridDim.y) {
        double acc = out[i + e * Nref];
        for (int64_t q = ebeg[e]; q < ebeg[e + 1]; ++q) {
            const int64_t k = eid[q] - k0;
            if (k >= 0 && k < nk) acc += R[k * Nref + i] * ecoef[q];
        }
        out[i + e * Nref] = acc;
    }
}

void launch_eit_combine(int64_t Nref, int64_t ne, const int64_t* ebeg, const int64_t* eid, const double* ecoef,
                        int64_t k0, int64_t nk, const double* R, double* out, cudaStream_t s) {
    if (ne == 0 || Nref == 0) return;
    ProfScope prof_("eit_combine", s);
    dim3 grid(nblocks(Nref, 256), (unsigned)std::min<int64_t>(ne, 32768));
    eit_combine_kernel<<<grid, 256, 0, s>>>(Nref, ne, ebeg, eid, ecoef, k0, nk, R, out);
    check_launch("EIT combine");
}

// ---------------------------------------------------------------------------
// Shared vertices.  Assembly runs on per-mesh vertex copies (every mesh keeps
// its own vertices, so each block kernel sees a contiguous range); the
// reference's unknowns are the distinct vertices.  With P the copy -> distinct
// vertex map, the reference's head matrix is P^T H P (its N block adds the
// cross-mesh term of a vertex shared by two meshes once with factor 1/2, which
// is the two symmetric copy entries with factor 1/4), its source rows are P^T
// times the copies' rows.  gbeg/gcopy: for distinct vertex u, its copies.
// Internal positions: triangles (and padding) i < nP are their own copies;
// vertex u sits at nP + u (distinct) or nP + v (copy).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void copies_of(int64_t i, int64_t nP, const int64_t* gbeg, const int64_t* gcopy,
                                          int64_t& k0, int64_t& k1) {
    if (i < nP) {
        k0 = -1 - i;   // encodes the single copy i
        k1 = k0 + 1;
    } else {
        k0 = gbeg[i - nP];
        k1 = gbeg[i - nP + 1];
    }
}
__device__ __forceinline__ int64_t copy_at(int64_t k, int64_t nP, const int64_t* gcopy) {
    return k < 0 ? -1 - k : nP + gcopy[k];
}

// Hg (lower triangle, Ng x Ng) = P^T Hl P from the lower triangle of Hl (symmetric).
__global__ void fold_hm_kernel(int64_t Ng, int64_t nP, const int64_t* __restrict__ gbeg,
                               const int64_t* __restrict__ gcopy, const double* __restrict__ hl, int64_t ldl,
                               double* hg, int64_t ldg) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= Ng) return;
    int64_t a0, a1;
    copies_of(i, nP, gbeg, gcopy, a0, a1);
    for (int64_t j = blockIdx.y; j <= i; j += gridDim.y) {
        int64_t b0, b1;
        copies_of(j, nP, gbeg, gcopy, b0, b1);
        double acc = 0.0;
        for (int64_t ka = a0; ka < a1; ++ka) {
            const int64_t a = copy_at(ka, nP, gcopy);
            for (int64_t kb = b0; kb < b1; ++kb) acc += hl[lower_at(a, copy_at(kb, nP, gcopy), ldl)];
        }
        hg[i + j * ldg] = acc;
    }
}

// out (Ng x ncol) = P^T in (Nl x ncol): rows of the copies summed.
__global__ void fold_rows_kernel(int64_t Ng, int64_t nP, const int64_t* __restrict__ gbeg,
                                 const int64_t* __restrict__ gcopy, int64_t ncol, const double* __restrict__ in,
                                 int64_t ldi, double* out, int64_t ldo) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= Ng) return;
    int64_t a0, a1;
    copies_of(i, nP, gbeg, gcopy, a0, a1);
    for (int64_t c = blockIdx.y; c < ncol; c += gridDim.y) {
        double acc = 0.0;
        for (int64_t k = a0; k < a1; ++k) acc += in[copy_at(k, nP, gcopy) + c * ldi];
        out[i + c * ldo] = acc;
    }
}

void launch_fold_hm(int64_t Ng, int64_t nP, const int64_t* gbeg, const int64_t* gcopy, const double* hl, int64_t ldl,
                    double* hg, int64_t ldg, cudaStream_t s) {
    ProfScope prof_("fold", s);
    dim3 grid(nblocks(Ng, 256), (unsigned)std::min<int64_t>(Ng, 32768));
    fold_hm_kernel<<<grid, 256, 0, s>>>(Ng, nP, gbeg, gcopy, hl, ldl, hg, ldg);
    check_launch("fold head matrix");
}

void launch_fold_rows(int64_t Ng, int64_t nP, const int64_t* gbeg, const int64_t* gcopy, int64_t ncol, const double* in,
                      int64_t ldi, double* out, int64_t ldo, cudaStream_t s) {
    if (ncol <= 0) return;
    ProfScope prof_("fold", s);
    dim3 grid(nblocks(Ng, 256), (unsigned)std::min<int64_t>(ncol, 32768));
    fold_rows_kernel<<<grid, 256, 0, s>>>(Ng, nP, gbeg, gcopy, ncol, in, ldi, out, ldo);
    check_launch("fold rows");
}

// out[r * rs + c * cs] (reference numbering r < Nref: distinct vertices, then
// triangle unknowns) = sum over the copies of unknown r of in[copy + c * ldi]
// (internal copy numbering).
__global__ void fold_to_reference_kernel(int64_t Nref, int64_t nvg, int64_t nP, const int64_t* __restrict__ gbeg,
                                         const int64_t* __restrict__ gcopy, int64_t ncol,
                                         const double* __restrict__ in, int64_t ldi, double* out, int64_t rs,
                                         int64_t cs) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= Nref) return;
    const int64_t i = r < nvg ? nP + r : r - nvg;
    int64_t a0, a1;
    copies_of(i, nP, gbeg, gcopy, a0, a1);
    for (int64_t c = blockIdx.y; c < ncol; c += gridDim.y) {
        double acc = 0.0;
        for (int64_t k = a0; k < a1; ++k) acc += in[copy_at(k, nP, gcopy) + c * ldi];
        out[r * rs + c * cs] = acc;
    }
}

// Columns of a per-copy matrix (nrow x (nv + triangles): vertex copies, then the triangle unknowns) folded to
// the reference's columns (distinct vertices, then triangles): out(:, r) = sum of the copies of vertex r, in
// copy order, for r < nvg; the triangle columns moved.
__global__ void fold_columns_kernel(int64_t nrow, int64_t Nref, int64_t nvg, int64_t nv, const int64_t* __restrict__ gbeg,
                                    const int64_t* __restrict__ gcopy, const double* __restrict__ in, int64_t ldi,
                                    double* out, int64_t ldo) {
    for (int64_t r = blockIdx.y; r < Nref; r += gridDim.y)
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nrow;
             i += (int64_t)gridDim.x * blockDim.x) {
            double acc = 0.0;
            if (r < nvg) {
                for (int64_t k = gbeg[r]; k < gbeg[r + 1]; ++k) acc += in[i + gcopy[k] * ldi];
            } else {
                acc = in[i + (r - nvg + nv) * ldi];
            }
            out[i + r * ldo] = acc;
        }
}

void launch_fold_columns(int64_t nrow, int64_t Nref, int64_t nvg, int64_t nv, const int64_t* gbeg,
                         const int64_t* gcopy, const double* in, int64_t ldi, double* out, int64_t ldo,
                         cudaStream_t s) {
    if (nrow <= 0) return;
    ProfScope prof_("fold", s);
    dim3 grid(nblocks(nrow, 256), (unsigned)std::min<int64_t>(Nref, 32768));
    fold_columns_kernel<<<grid, 256, 0, s>>>(nrow, Nref, nvg, nv, gbeg, gcopy, in, ldi, out, ldo);
    check_launch("fold columns");
}

void launch_fold_to_reference(int64_t Nref, int64_t nvg, int64_t nP, const int64_t* gbeg, const int64_t* gcopy,
                              int64_t ncol, const double* in, int64_t ldi, double* out, int64_t rs, int64_t cs,
                              cudaStream_t s) {
    if (ncol <= 0) return;
    ProfScope prof_("fold", s);
    dim3 grid(nblocks(Nref, 256), (unsigned)std::min<int64_t>(ncol, 32768));
    fold_to_reference_kernel<<<grid, 256, 0, s>>>(Nref, nvg, nP, gbeg, gcopy, ncol, in, ldi, out, rs, cs);
    check_launch("fold to reference");
}

}  // namespace omg
