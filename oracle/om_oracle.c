/*
 * om_oracle.c -- CPU restatement of OpenMEEG's symmetric-BEM forward path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker and the CPU
 * baseline ("port"); the product never links or calls it.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU legs load it.
 *
 * Each routine restates the reference algorithm it cites (paths are relative
 * to the OpenMEEG source tree).  Storage follows the reference SymMatrix:
 * packed upper, column-major, entry (i,j), i<=j, at i + j*(j+1)/2
 * (OpenMEEGMaths/include/symmatrix.h:52-62).  Indices are 64-bit.
 *
 * Geometry arrives pre-digested (unknown numbering, mesh pairs, coefficients,
 * deflation parts) from oracle/oracle.py, which restates the Geometry logic.
 *
 * Build (oracle.py build()): gcc -O2 -ffp-contract=off -fopenmp -fPIC -shared -std=c11 om_oracle.c -lm.
 * With contraction off the arithmetic is the reference's own (no fused multiply-adds)
 * on x86 and Arm hosts alike.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OO_K (1.0 / (4.0 * M_PI))      /* OpenMEEG/include/constants.h:23 */
#define OO_MAGFACTOR 1e-7              /* OpenMEEG/include/constants.h:22 */

/* ------------------------------------------------------------------------ */
/* Small vector helpers                                                      */
/* ------------------------------------------------------------------------ */
typedef struct { double x, y, z; } v3;
static inline v3 vsub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline v3 vadd(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static inline v3 vscale(v3 a, double s) { v3 r = {a.x * s, a.y * s, a.z * s}; return r; }
static inline double vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double vnorm(v3 a) { return sqrt(vdot(a, a)); }
static inline v3 vcross(v3 a, v3 b) {
    v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return r;
}

/* ------------------------------------------------------------------------ */
/* Triangle: normal/area (triangle.h:57-62), solid angle (triangle.h:123-136) */
/* ------------------------------------------------------------------------ */
typedef struct {
    v3 p[3];
    v3 n;
    double area;
} tri_t;

static void tri_make(tri_t* t, v3 a, v3 b, v3 c) {
    t->p[0] = a; t->p[1] = b; t->p[2] = c;
    v3 nn = vcross(vsub(b, a), vsub(c, a));
    double nrm = vnorm(nn);
    t->area = 0.5 * nrm;
    t->n = vscale(nn, 1.0 / nrm);
}

static double tri_solid_angle(const tri_t* t, v3 V) {
    v3 r0 = vsub(t->p[0], V), r1 = vsub(t->p[1], V), r2 = vsub(t->p[2], V);
    double d0 = vnorm(r0), d1 = vnorm(r1), d2 = vnorm(r2);
    double pr0 = vdot(r1, r2), pr1 = vdot(r2, r0), pr2 = vdot(r0, r1);
    double prod = d0 * d1 * d2;
    double d = 2 * t->area * vdot(r0, t->n);
    return (fabs(d) < 1e-10) ? 0.0 : 2 * atan2(d, prod + (d0 * pr0 + d1 * pr1 + d2 * pr2));
}

/* ------------------------------------------------------------------------ */
/* Analytic kernels (analytics.h)                                            */
/* ------------------------------------------------------------------------ */
static const int NEXT[3] = {1, 2, 0};

/* OperatorS (analytics.h:19-67): closed form of int_T 1/|y-x| dy. */
typedef struct {
    const tri_t* t;
    double len[3];
    v3 en[3];
} opS_t;

static void opS_make(opS_t* s, const tri_t* t) {
    s->t = t;
    for (int i = 0; i < 3; ++i) {
        v3 vref = vsub(t->p[i], t->p[NEXT[i]]);
        double len = vnorm(vref);
        v3 unit = vscale(vref, 1.0 / len);
        s->len[i] = len;
        s->en[i] = vcross(t->n, unit);
    }
}

static double opS_eval(const opS_t* s, v3 x) {
    const tri_t* t = s->t;
    v3 r[3] = {vsub(t->p[0], x), vsub(t->p[1], x), vsub(t->p[2], x)};
    double d[3] = {vnorm(r[0]), vnorm(r[1]), vnorm(r[2])};
    double R[3] = {d[0] + d[1], d[1] + d[2], d[2] + d[0]};
    double sum = 0.0;
    for (int i = 0; i < 3; ++i) sum += vdot(r[i], s->en[i]) * atanh(s->len[i] / R[i]);
    return 2 * sum - vdot(r[0], t->n) * tri_solid_angle(t, x);
}

/* P1SingleLayerPotential (analytics.h:75-128): 3 P1-weighted D-kernel integrals. */
typedef struct {
    const tri_t* t;
    v3 D[3], U[3];
} p1_t;

static void p1_make(p1_t* s, const tri_t* t) {
    s->t = t;
    s->D[0] = vsub(t->p[1], t->p[0]);
    s->D[1] = vsub(t->p[2], t->p[1]);
    s->D[2] = vsub(t->p[0], t->p[2]);
    for (int i = 0; i < 3; ++i) s->U[i] = vscale(s->D[i], 1.0 / vnorm(s->D[i]));
}

static v3 p1_eval(const p1_t* s, v3 x) {
    const tri_t* t = s->t;
    v3 r[3] = {vsub(t->p[0], x), vsub(t->p[1], x), vsub(t->p[2], x)};
    double d[3] = {vnorm(r[0]), vnorm(r[1]), vnorm(r[2])};
    v3 Z[3] = {vcross(r[1], r[2]), vcross(r[2], r[0]), vcross(r[0], r[1])};
    double pr[3] = {vdot(r[1], r[2]), vdot(r[2], r[0]), vdot(r[0], r[1])};
    v3 n = t->n;
    double h = vdot(r[0], n);
    double dd = 2 * h * t->area;
    v3 zero = {0, 0, 0};
    if (fabs(h) < 1e-10) return zero;
    v3 S = zero;
    for (int i = 0; i < 3; ++i) {
        int i1 = NEXT[i];
        double lg = log((d[i1] + vdot(r[i1], s->U[i])) / (d[i] + vdot(r[i], s->U[i])));
        S = vadd(S, vscale(s->U[i], lg));
    }
    double d1 = d[0] * d[1] * d[2] + (d[0] * pr[0] + d[1] * pr[1] + d[2] * pr[2]);
    double omega = atan2(dd, d1);
    v3 E1 = {vdot(Z[0], n), vdot(Z[1], n), vdot(Z[2], n)};
    v3 E2 = {vdot(s->D[1], S), vdot(s->D[2], S), vdot(s->D[0], S)};
    v3 res = vadd(vscale(E1, omega), vscale(E2, 0.5 * h));
    return vscale(res, 1.0 / t->area);
}

/* ------------------------------------------------------------------------ */
/* Quadrature (integrator.h:44-160).  Dunavant/Bonnet rules with 3/6/7/16    */
/* points; the tabulated digits must match the reference's exactly for       */
/* 1e-10 parity.                                                             */
/* ------------------------------------------------------------------------ */
static const int NBPTS[4] = {3, 6, 7, 16};
static const double RULES[4][16][4] = {
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

typedef struct {
    int order;      /* 0..3 -> 3,6,7,16 points (integrator.h:254) */
    int levels;     /* adaptive depth (0 = plain rule) */
    double tol;     /* relative tolerance of the adaptive test */
} oo_integrator;

/* A vector-valued integrand with up to 3 components (dim = 1 or 3). */
typedef void (*integrand_fn)(const void* ctx, v3 x, double* out);

static void rule_integrate(integrand_fn f, const void* ctx, int dim, const v3 P[3], double area, int order,
                           double* res) {
    double acc[3] = {0, 0, 0};
    for (int q = 0; q < NBPTS[order]; ++q) {
        const double* r = RULES[order][q];
        v3 v = {0, 0, 0};
        for (int j = 0; j < 3; ++j) v = vadd(v, vscale(P[j], r[j]));
        double val[3];
        f(ctx, v, val);
        for (int c = 0; c < dim; ++c) acc[c] += r[3] * val[c];
    }
    for (int c = 0; c < dim; ++c) res[c] = area * acc[c];
}

static double vnorm_dim(const double* a, int dim) {
    if (dim == 1) return fabs(a[0]);
    return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
}

/* adaptive_integration (integrator.h:228-252) */
static void adaptive_integrate(integrand_fn f, const void* ctx, int dim, const v3 P[3], double area,
                               const double* coarse, int level, const oo_integrator* I, double* out) {
    v3 mid[3] = {vscale(vadd(P[1], P[2]), 0.5), vscale(vadd(P[2], P[0]), 0.5), vscale(vadd(P[0], P[1]), 0.5)};
    v3 NT[4][3] = {{P[0], mid[1], mid[2]}, {mid[0], P[1], mid[2]}, {mid[0], mid[1], P[2]}, {mid[0], mid[1], mid[2]}};
    double sub_area = 0.25 * area;
    double refined[3] = {0, 0, 0}, integ[4][3];
    for (int i = 0; i < 4; ++i) {
        rule_integrate(f, ctx, dim, NT[i], sub_area, I->order, integ[i]);
        for (int c = 0; c < dim; ++c) refined[c] += integ[i][c];
    }
    double diff[3];
    for (int c = 0; c < dim; ++c) diff[c] = coarse[c] - refined[c];
    if (vnorm_dim(diff, dim) <= I->tol * vnorm_dim(coarse, dim) || level == 0) {
        for (int c = 0; c < dim; ++c) out[c] = refined[c];
        return;
    }
    double sum[3] = {0, 0, 0};
    for (int i = 0; i < 4; ++i) {
        double part[3];
        adaptive_integrate(f, ctx, dim, NT[i], sub_area, integ[i], level - 1, I, part);
        for (int c = 0; c < dim; ++c) sum[c] += part[c];
    }
    for (int c = 0; c < dim; ++c) out[c] = sum[c];
}

/* Integrator::integrate (integrator.h:44-48) */
static void integrate(integrand_fn f, const void* ctx, int dim, const tri_t* t, const oo_integrator* I, double* out) {
    double coarse[3];
    rule_integrate(f, ctx, dim, t->p, t->area, I->order, coarse);
    if (I->levels == 0) {
        for (int c = 0; c < dim; ++c) out[c] = coarse[c];
        return;
    }
    adaptive_integrate(f, ctx, dim, t->p, t->area, coarse, I->levels, I, out);
}

static void f_opS(const void* ctx, v3 x, double* out) { out[0] = opS_eval((const opS_t*)ctx, x); }
static void f_p1(const void* ctx, v3 x, double* out) {
    v3 r = p1_eval((const p1_t*)ctx, x);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

/* ------------------------------------------------------------------------ */
/* Flat geometry descriptor                                                  */
/* ------------------------------------------------------------------------ */
typedef struct {
    int64_t nv;               /* vertices (all meshes) */
    const double* V;          /* nv x 3 */
    int64_t nt;               /* triangles (all meshes) */
    const int64_t* T;         /* nt x 3, global vertex ids */
    int nmesh;
    const int64_t* mesh_vbeg; /* nmesh+1: vertices of mesh m are [vbeg[m], vbeg[m+1]) */
    const int64_t* mesh_tbeg; /* nmesh+1 */
    const int64_t* vidx;      /* unknown index of each vertex */
    const int64_t* tidx;      /* unknown index of each triangle (may be >= N for barrier meshes) */
    const int* barrier;       /* per mesh: current barrier flag */
    int npairs;
    const int* pairs;         /* npairs x 2 (m1, m2) in reference order */
    const double* coefs;      /* npairs x 3 (S, N, D) */
    int nparts;
    const int* part_beg;      /* nparts+1 offsets into part_meshes */
    const int* part_meshes;   /* outermost meshes of each part, in part order */
    int64_t N;                /* HeadMat size */
} oo_geom;

/* vertex -> incident triangles (mesh.h:252-257), in triangle order */
typedef struct {
    int64_t* beg;   /* nv+1 */
    int64_t* tri;   /* incidence list */
} v2t_t;

static void build_v2t(const oo_geom* g, v2t_t* a) {
    a->beg = (int64_t*)calloc((size_t)g->nv + 1, sizeof(int64_t));
    for (int64_t t = 0; t < g->nt; ++t)
        for (int j = 0; j < 3; ++j) a->beg[g->T[3 * t + j] + 1]++;
    for (int64_t v = 0; v < g->nv; ++v) a->beg[v + 1] += a->beg[v];
    a->tri = (int64_t*)malloc(sizeof(int64_t) * (size_t)(a->beg[g->nv] + 1));
    int64_t* fill = (int64_t*)calloc((size_t)g->nv, sizeof(int64_t));
    for (int64_t t = 0; t < g->nt; ++t)
        for (int j = 0; j < 3; ++j) {
            int64_t v = g->T[3 * t + j];
            a->tri[a->beg[v] + fill[v]++] = t;
        }
    free(fill);
}

static void free_v2t(v2t_t* a) { free(a->beg); free(a->tri); }

static inline int64_t pk(int64_t i, int64_t j) {
    if (i > j) { int64_t k = i; i = j; j = k; }
    return i + j * (j + 1) / 2;
}

static void make_tri(const oo_geom* g, int64_t t, tri_t* out) {
    const int64_t* tt = g->T + 3 * t;
    v3 a = {g->V[3 * tt[0]], g->V[3 * tt[0] + 1], g->V[3 * tt[0] + 2]};
    v3 b = {g->V[3 * tt[1]], g->V[3 * tt[1] + 1], g->V[3 * tt[1] + 2]};
    v3 c = {g->V[3 * tt[2]], g->V[3 * tt[2] + 1], g->V[3 * tt[2] + 2]};
    tri_make(out, a, b, c);
}

/* Local position of vertex v in triangle t. */
static int local_index(const oo_geom* g, int64_t t, int64_t v) {
    for (int j = 0; j < 3; ++j) if (g->T[3 * t + j] == v) return j;
    return -1;
}

/* CB vector of Edge(V) (triangle.h:87-94,154): vertex(e0) - vertex(e1). */
static v3 edge_cb(const tri_t* T, int li) {
    static const int IDX[3][2] = {{1, 2}, {2, 0}, {0, 1}};
    return vsub(T->p[IDX[li][0]], T->p[IDX[li][1]]);
}

/* ------------------------------------------------------------------------ */
/* HeadMat (assembleHeadMat.cpp:73-115, operators.h:155-485)                 */
/* ------------------------------------------------------------------------ */

/* S block into a callback-addressed store. mode 0: into HM (packed), with
 * diagonal block upper-only; mode 1: into a temporary dense block [n1 x n2]. */
static void S_block(const oo_geom* g, const tri_t* tris, int m1, int m2, double coeff, const oo_integrator* I,
                    double* hm, double* tmp) {
    const int64_t t1b = g->mesh_tbeg[m1], t1e = g->mesh_tbeg[m1 + 1];
    const int64_t t2b = g->mesh_tbeg[m2], t2e = g->mesh_tbeg[m2 + 1];
    const int64_t n2 = t2e - t2b;
    const int same = (m1 == m2);
    #pragma omp parallel for schedule(dynamic, 4)
    for (int64_t t1 = t1b; t1 < t1e; ++t1) {
        opS_t S;
        opS_make(&S, &tris[t1]);
        for (int64_t t2 = same ? t1 : t2b; t2 < t2e; ++t2) {
            double val;
            integrate(f_opS, &S, 1, &tris[t2], I, &val);
            val *= coeff;
            if (hm) hm[pk(g->tidx[t1], g->tidx[t2])] = val;
            else {
                tmp[(t1 - t1b) * n2 + (t2 - t2b)] = val;
                if (same) tmp[(t2 - t2b) * n2 + (t1 - t1b)] = val;
            }
        }
    }
}

/* N from S (operators.h:119-148, 271-296, 454-480). */
static double N_entry(const oo_geom* g, const tri_t* tris, const v2t_t* a, double factor, int64_t v1, int64_t v2,
                      int m1, int m2, const double* hm, double hm_scale, const double* tmp) {
    const int64_t t1b = g->mesh_tbeg[m1], t1e = g->mesh_tbeg[m1 + 1];
    const int64_t t2b = g->mesh_tbeg[m2], t2e = g->mesh_tbeg[m2 + 1];
    const int64_t n2 = t2e - t2b;
    double result = 0.0;
    for (int64_t k1 = a->beg[v1]; k1 < a->beg[v1 + 1]; ++k1) {
        int64_t tp1 = a->tri[k1];
        if (tp1 < t1b || tp1 >= t1e) continue;
        v3 CB1 = edge_cb(&tris[tp1], local_index(g, tp1, v1));
        for (int64_t k2 = a->beg[v2]; k2 < a->beg[v2 + 1]; ++k2) {
            int64_t tp2 = a->tri[k2];
            if (tp2 < t2b || tp2 >= t2e) continue;
            v3 CB2 = edge_cb(&tris[tp2], local_index(g, tp2, v2));
            double s = hm ? hm[pk(g->tidx[tp1], g->tidx[tp2])] * hm_scale : tmp[(tp1 - t1b) * n2 + (tp2 - t2b)];
            result -= factor * vdot(CB1, CB2) * s / (tris[tp1].area * tris[tp2].area);
        }
    }
    return result;
}

static void N_block(const oo_geom* g, const tri_t* tris, const v2t_t* a, int m1, int m2, double coeff,
                    double* hm, const double* Ssrc_hm, const double* tmp) {
    const int64_t v1b = g->mesh_vbeg[m1], v1e = g->mesh_vbeg[m1 + 1];
    const int64_t v2b = g->mesh_vbeg[m2], v2e = g->mesh_vbeg[m2 + 1];
    const int same = (m1 == m2);
    #pragma omp parallel for schedule(dynamic, 4)
    for (int64_t v1 = v1b; v1 < v1e; ++v1) {
        int64_t end = same ? v1 + 1 : v2e;
        for (int64_t v2 = v2b; v2 < end; ++v2) {
            double factor = same ? 0.25 : ((v1 == v2) ? 0.5 : 0.25);
            double n = N_entry(g, tris, a, factor, v1, v2, m1, m2, Ssrc_hm, 1.0, tmp);
            hm[pk(g->vidx[v1], g->vidx[v2])] += n * coeff;
        }
    }
}

/* BlocksBase::D (operators.h:83-115): mat(t1, vertex_i(t2)) += coeff * int_t1 P1SLP(t2)_i */
static void D_block(const oo_geom* g, const tri_t* tris, int ma, int mb, double coeff, const oo_integrator* I,
                    double* hm) {
    const int64_t tab = g->mesh_tbeg[ma], tae = g->mesh_tbeg[ma + 1];
    const int64_t tbb = g->mesh_tbeg[mb], tbe = g->mesh_tbeg[mb + 1];
    #pragma omp parallel for schedule(dynamic, 4)
    for (int64_t t1 = tab; t1 < tae; ++t1) {
        for (int64_t t2 = tbb; t2 < tbe; ++t2) {
            p1_t P;
            p1_make(&P, &tris[t2]);
            double tot[3];
            integrate(f_p1, &P, 3, &tris[t1], I, tot);
            for (int i = 0; i < 3; ++i) hm[pk(g->tidx[t1], g->vidx[g->T[3 * t2 + i]])] += tot[i] * coeff;
        }
    }
}

/* Fills `hm` (packed upper, N(N+1)/2 doubles) with the HeadMat. */
int oo_headmat(const oo_geom* g, const oo_integrator* I, double* hm) {
    const int64_t N = g->N;
    memset(hm, 0, sizeof(double) * (size_t)(N * (N + 1) / 2));
    tri_t* tris = (tri_t*)malloc(sizeof(tri_t) * (size_t)g->nt);
    for (int64_t t = 0; t < g->nt; ++t) make_tri(g, t, &tris[t]);
    v2t_t a;
    build_v2t(g, &a);
    for (int p = 0; p < g->npairs; ++p) {
        const int m1 = g->pairs[2 * p], m2 = g->pairs[2 * p + 1];
        const double cS = g->coefs[3 * p], cN = g->coefs[3 * p + 1], cD = g->coefs[3 * p + 2];
        const int same = (m1 == m2);
        /* set_S_block (operators.h:179-185, 363-369) */
        double Scoeff = 0.0;
        if (same ? !g->barrier[m1] : (!g->barrier[m1] && !g->barrier[m2])) {
            S_block(g, tris, m1, m2, cS, I, hm, NULL);
            Scoeff = cS;
        }
        /* set_N_block (operators.h:239-248, 427-436) */
        if (Scoeff != 0.0) {
            N_block(g, tris, &a, m1, m2, cN / Scoeff, hm, hm, NULL);
        } else {
            int64_t n1 = g->mesh_tbeg[m1 + 1] - g->mesh_tbeg[m1];
            int64_t n2 = g->mesh_tbeg[m2 + 1] - g->mesh_tbeg[m2];
            double* tmp = (double*)malloc(sizeof(double) * (size_t)(n1 * n2));
            S_block(g, tris, m1, m2, 1.0, I, NULL, tmp);
            N_block(g, tris, &a, m1, m2, cN, hm, NULL, tmp);
            free(tmp);
        }
        /* set_D_block / set_Dstar_block (operators.h:190-197, 374-384) */
        if (!g->barrier[m1]) D_block(g, tris, m1, m2, cD, I, hm);
        if (!same && !g->barrier[m2]) D_block(g, tris, m2, m1, cD, I, hm);
    }
    /* deflate (assembleHeadMat.cpp:27-60) */
    for (int q = 0; q < g->nparts; ++q) {
        int64_t nb = 0, i_first = 0;
        for (int k = g->part_beg[q]; k < g->part_beg[q + 1]; ++k) {
            int m = g->part_meshes[k];
            nb += g->mesh_vbeg[m + 1] - g->mesh_vbeg[m];
            if (i_first == 0) i_first = g->vidx[g->mesh_vbeg[m]];
        }
        const double coef = hm[pk(i_first, i_first)] / (double)nb;
        for (int k = g->part_beg[q]; k < g->part_beg[q + 1]; ++k) {
            int m = g->part_meshes[k];
            for (int64_t v1 = g->mesh_vbeg[m]; v1 < g->mesh_vbeg[m + 1]; ++v1)
                for (int64_t v2 = v1; v2 < g->mesh_vbeg[m + 1]; ++v2) hm[pk(g->vidx[v1], g->vidx[v2])] += coef;
        }
    }
    free_v2t(&a);
    free(tris);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* DipSourceMat (assembleSourceMat.cpp:66-104, operators.cpp:40-88)          */
/* ------------------------------------------------------------------------ */
typedef struct { v3 r0, q; } dip_t;

/* Dipole::potential (dipole.h:29-36) */
static double dip_potential(const dip_t* d, v3 r) {
    v3 x = vsub(r, d->r0);
    double nrm2 = vdot(x, x);
    return vdot(d->q, x) / (nrm2 * sqrt(nrm2));
}
/* Dipole::gradient (dipole.h:38-46) */
static double dip_gradient(const dip_t* d, v3 r, v3 n) {
    v3 x = vsub(r, d->r0);
    double inv = 1.0 / vdot(x, x);
    v3 grad = vsub(d->q, vscale(x, 3 * vdot(d->q, x) * inv));
    return vdot(grad, n) * (inv * sqrt(inv));
}

typedef struct { const dip_t* d; const tri_t* t; double d11, d12, d22; v3 e10, e20; } pd_t;

/* BarycentricCoordinates (BarycentricCoordinates.h:33-69) */
static void pd_make(pd_t* s, const dip_t* d, const tri_t* t) {
    s->d = d; s->t = t;
    s->e10 = vsub(t->p[1], t->p[0]);
    s->e20 = vsub(t->p[2], t->p[0]);
    double c11 = vdot(s->e10, s->e10), c12 = vdot(s->e10, s->e20), c22 = vdot(s->e20, s->e20);
    double inv_det = 1.0 / (c11 * c22 - c12 * c12);
    s->d11 = c22 * inv_det; s->d12 = -c12 * inv_det; s->d22 = c11 * inv_det;
}

/* PotentialDerivative (analytics.h:140-150) */
static void f_potderiv(const void* ctx, v3 r, double* out) {
    const pd_t* s = (const pd_t*)ctx;
    v3 v = vsub(r, s->t->p[0]);
    double d1 = vdot(v, s->e10), d2 = vdot(v, s->e20);
    double l1 = s->d11 * d1 + s->d12 * d2;
    double l2 = s->d12 * d1 + s->d22 * d2;
    double l0 = 1.0 - l1 - l2;
    double g = dip_gradient(s->d, r, s->t->n);
    out[0] = g * l0; out[1] = g * l1; out[2] = g * l2;
}
static void f_pot(const void* ctx, v3 r, double* out) { out[0] = dip_potential(((const pd_t*)ctx)->d, r); }

/* One DSM column for a dipole whose domain boundary is described by
 * (bmesh[k], bcoeffD[k]) k<nb and domain conductivity `cond`.  The column is
 * accumulated in `col` (length N). */
static void dsm_column(const oo_geom* g, const tri_t* tris, const dip_t* d, int nb, const int* bmesh,
                       const double* bcoeffD, double cond, const oo_integrator* I, double* col) {
    for (int k = 0; k < nb; ++k) {
        int m = bmesh[k];
        double coeffD = bcoeffD[k];
        for (int64_t t = g->mesh_tbeg[m]; t < g->mesh_tbeg[m + 1]; ++t) {
            pd_t s;
            pd_make(&s, d, &tris[t]);
            double v[3];
            integrate(f_potderiv, &s, 3, &tris[t], I, v);
            for (int j = 0; j < 3; ++j) col[g->vidx[g->T[3 * t + j]]] += v[j] * coeffD;
        }
        if (!g->barrier[m]) {
            double coeff = coeffD / cond;
            for (int64_t t = g->mesh_tbeg[m]; t < g->mesh_tbeg[m + 1]; ++t) {
                pd_t s;
                pd_make(&s, d, &tris[t]);
                double v;
                integrate(f_pot, &s, 1, &tris[t], I, &v);
                col[g->tidx[t]] += v * coeff;
            }
        }
    }
}

/* DSM for ndip dipoles (ndip x 6, row-major x y z qx qy qz).  For each
 * dipole, dom_nb[i] boundary meshes listed in dom_mesh[i*maxb ...] with
 * coefficients dom_coeff[...] and domain conductivity dom_cond[i]
 * (assembleSourceMat.cpp:79-98); dom_nb[i]==0 or cond==0 leaves the column
 * zero.  Output `out` is N x ndip column-major. */
int oo_dsm(const oo_geom* g, const double* dip, int64_t ndip, const int* dom_nb, const int* dom_mesh,
           const double* dom_coeff, const double* dom_cond, int maxb, const oo_integrator* I, double* out) {
    const int64_t N = g->N;
    tri_t* tris = (tri_t*)malloc(sizeof(tri_t) * (size_t)g->nt);
    for (int64_t t = 0; t < g->nt; ++t) make_tri(g, t, &tris[t]);
    memset(out, 0, sizeof(double) * (size_t)(N * ndip));
    #pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < ndip; ++i) {
        dip_t d = {{dip[6 * i], dip[6 * i + 1], dip[6 * i + 2]}, {dip[6 * i + 3], dip[6 * i + 4], dip[6 * i + 5]}};
        if (dom_nb[i] == 0 || dom_cond[i] == 0.0) continue;
        dsm_column(g, tris, &d, dom_nb[i], dom_mesh + (size_t)i * maxb, dom_coeff + (size_t)i * maxb, dom_cond[i],
                   I, out + (size_t)i * N);
    }
    free(tris);
    return 0;
}

/* Surf2VolMat (assembleHeadMat.cpp:325-363) through PartialBlock::addD and
 * PartialBlock::S (operators.h:302-331).  Point i (already kept: conducting
 * domain) sees the boundary meshes mesh[i*maxb + k], k < nb[i], each with
 * c = K * mesh_orientation (domain.h:43-45):
 *   out(i, vertex unknowns) += -c * P1SingleLayerPotential(triangle)(x)
 *   out(i, triangle unknown)  =  c / cond * OperatorS(triangle)(x)   (no barrier)
 * out is np x N, column-major. */
int oo_surf2vol(const oo_geom* g, const double* pts, int64_t np, const int* nb, const int* mesh,
                const double* coeff, const double* cond, int maxb, double* out) {
    tri_t* tris = (tri_t*)malloc(sizeof(tri_t) * (size_t)g->nt);
    for (int64_t t = 0; t < g->nt; ++t) make_tri(g, t, &tris[t]);
    memset(out, 0, sizeof(double) * (size_t)(np * g->N));
    #pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < np; ++i) {
        v3 x = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        for (int k = 0; k < nb[i]; ++k) {
            const int m = mesh[(size_t)i * maxb + k];
            const double c = coeff[(size_t)i * maxb + k];
            for (int64_t t = g->mesh_tbeg[m]; t < g->mesh_tbeg[m + 1]; ++t) {
                p1_t P;
                p1_make(&P, &tris[t]);
                const v3 I = p1_eval(&P, x);
                const double Ij[3] = {I.x, I.y, I.z};
                for (int j = 0; j < 3; ++j) out[i + np * g->vidx[g->T[3 * t + j]]] += Ij[j] * -c;
                if (!g->barrier[m]) {
                    opS_t S;
                    opS_make(&S, &tris[t]);
                    out[i + np * g->tidx[t]] = c / cond[i] * opS_eval(&S, x);
                }
            }
        }
    }
    free(tris);
    return 0;
}

/* Rows of the EITSourceMat transfer matrix (assembleSourceMat.cpp:115-134) for
 * the triangles tri[0..n): for each communicating pair (mesh1, mesh2) whose
 * mesh1 holds the triangle and is a current barrier,
 *   D:  row(vertex of t2 in mesh2) += cD[p] * integral over t of P1SingleLayerPotential(t2)
 *   Id: row(vertex of t) += -1/2 * area(t) / 3                  (mesh1 == mesh2)
 *   S:  row(triangle unknown of t2) = cS[p] * integral over t2 of OperatorS(t)   (mesh1 != mesh2)
 * rows is n x N, row-major (only the N unknown columns are kept). */
int oo_eit_rows(const oo_geom* g, const int64_t* tri, int64_t n, const double* cD, const double* cS,
                const oo_integrator* I, double* rows) {
    const int64_t N = g->N;
    tri_t* tris = (tri_t*)malloc(sizeof(tri_t) * (size_t)g->nt);
    for (int64_t t = 0; t < g->nt; ++t) make_tri(g, t, &tris[t]);
    memset(rows, 0, sizeof(double) * (size_t)(n * N));
    #pragma omp parallel for schedule(dynamic, 1)
    for (int64_t k = 0; k < n; ++k) {
        const int64_t t = tri[k];
        int m1 = 0;
        while (t >= g->mesh_tbeg[m1 + 1]) ++m1;
        if (!g->barrier[m1]) continue;
        double* row = rows + (size_t)k * N;
        for (int p = 0; p < g->npairs; ++p) {
            if (g->pairs[2 * p] != m1) continue;
            const int m2 = g->pairs[2 * p + 1];
            for (int64_t t2 = g->mesh_tbeg[m2]; t2 < g->mesh_tbeg[m2 + 1]; ++t2) {
                p1_t P;
                p1_make(&P, &tris[t2]);
                double total[3];
                integrate(f_p1, &P, 3, &tris[t], I, total);
                for (int i = 0; i < 3; ++i) row[g->vidx[g->T[3 * t2 + i]]] += total[i] * cD[p];
            }
            if (m2 == m1) {
                for (int i = 0; i < 3; ++i) row[g->vidx[g->T[3 * t + i]]] += tris[t].area / 3.0 * -0.5;
            } else if (!g->barrier[m2]) {
                opS_t S;
                opS_make(&S, &tris[t]);
                for (int64_t t2 = g->mesh_tbeg[m2]; t2 < g->mesh_tbeg[m2 + 1]; ++t2) {
                    double v;
                    integrate(f_opS, &S, 1, &tris[t2], I, &v);
                    row[g->tidx[t2]] = v * cS[p];
                }
            }
        }
    }
    free(tris);
    return 0;
}

/* Total solid angle of each mesh seen from each point (Mesh::solid_angle,
 * mesh.cpp:239-244); out is npts x nmesh.  Used for Domain::contains. */
int oo_mesh_solid_angles(const oo_geom* g, const double* pts, int64_t npts, double* out) {
    tri_t* tris = (tri_t*)malloc(sizeof(tri_t) * (size_t)g->nt);
    for (int64_t t = 0; t < g->nt; ++t) make_tri(g, t, &tris[t]);
    #pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < npts; ++i) {
        v3 p = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        for (int m = 0; m < g->nmesh; ++m) {
            double s = 0.0;
            for (int64_t t = g->mesh_tbeg[m]; t < g->mesh_tbeg[m + 1]; ++t) s += tri_solid_angle(&tris[t], p);
            out[i * g->nmesh + m] = s;
        }
    }
    free(tris);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Head2EEGMat: nearest triangle by Danielsson (danielsson.cpp:26-128)       */
/* ------------------------------------------------------------------------ */
static double dpc(v3 p, const tri_t* T, double alphas[3], int nb, int idx[3], int* inside) {
    if (nb == 1) {
        alphas[idx[0]] = 1.0;
        return vnorm(vsub(p, T->p[idx[0]]));
    }
    v3 A0Ai[3];
    for (int i = 1; i < nb; ++i) A0Ai[i] = vsub(T->p[idx[i]], T->p[idx[0]]);
    v3 A0M = vsub(p, T->p[idx[0]]);
    if (nb == 2) {
        alphas[idx[1]] = vdot(A0M, A0Ai[1]) / vdot(A0Ai[1], A0Ai[1]);
        alphas[idx[0]] = 1.0 - alphas[idx[1]];
    } else {
        double a00 = vdot(A0Ai[1], A0Ai[1]), a10 = vdot(A0Ai[1], A0Ai[2]), a11 = vdot(A0Ai[2], A0Ai[2]);
        double b0 = vdot(A0M, A0Ai[1]), b1 = vdot(A0M, A0Ai[2]);
        double d = a00 * a11 - a10 * a10;
        alphas[idx[1]] = (b0 * a11 - b1 * a10) / d;
        alphas[idx[2]] = (a00 * b1 - a10 * b0) / d;
        alphas[idx[0]] = 1.0 - alphas[idx[1]] - alphas[idx[2]];
    }
    for (int i = 0; i < nb; ++i)
        if (alphas[idx[i]] < 0) {
            *inside = 0;
            alphas[idx[i]] = 0;
            int tmp = idx[i]; idx[i] = idx[nb - 1]; idx[nb - 1] = tmp;
            return dpc(p, T, alphas, nb - 1, idx, inside);
        }
    v3 MH = vscale(A0M, -1.0);
    for (int i = 1; i < nb; ++i) MH = vadd(MH, vscale(A0Ai[i], alphas[idx[i]]));
    return vnorm(MH);
}

/* For each electrode, the nearest triangle among the listed meshes
 * (meshes of interfaces bounding zero-conductivity domains, in
 * dist_point_geom order) and its 3 barycentric weights.  out_tri[i] is the
 * global triangle id, out_w[3i..3i+2] the weights of its vertices 0..2. */
int oo_h2em(const oo_geom* g, const double* pos, int64_t ne, int nm, const int* meshes, int64_t* out_tri,
            double* out_w) {
    /* dist_point_geom (danielsson.cpp:107-128) visits the interfaces in order;
     * each dist_point_interface call leaves the weights of its own nearest
     * triangle in the shared `alphas`, so the weights returned are those of the
     * last interface's nearest triangle, while the triangle is the overall
     * nearest (first strictly smaller distance). */
    #pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < ne; ++i) {
        v3 p = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        double best = 1.79769313486231570e+308;
        for (int k = 0; k < nm; ++k) {
            int m = meshes[k];
            double mbest = 1.79769313486231570e+308;
            int64_t mt = -1;
            double mw[3] = {0, 0, 0};
            for (int64_t t = g->mesh_tbeg[m]; t < g->mesh_tbeg[m + 1]; ++t) {
                tri_t T;
                make_tri(g, t, &T);
                double al[3] = {0, 0, 0};
                int idx[3] = {0, 1, 2}, inside = 1;
                double dist = dpc(p, &T, al, 3, idx, &inside);
                if (dist < mbest) {
                    mbest = dist;
                    mt = t;
                    mw[0] = al[0]; mw[1] = al[1]; mw[2] = al[2];
                }
            }
            if (mbest < best) {
                best = mbest;
                out_tri[i] = mt;
            }
            out_w[3 * i] = mw[0]; out_w[3 * i + 1] = mw[1]; out_w[3 * i + 2] = mw[2];
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Head2MEGMat (assembleSensors.cpp:69-96, assembleFerguson.cpp:18-31,       */
/* operators.cpp:17-38, operators.h:40-61).  Output: nsens x N column-major, */
/* nonzero on vertex columns only.  jump[m] = conductivity jump of mesh m.   */
/* Sensor weights (sensors.h:191-196) are applied by the caller.             */
/* ------------------------------------------------------------------------ */
int oo_h2mm(const oo_geom* g, const double* pos, const double* ori, int64_t np, const double* jump, double* out) {
    tri_t* tris = (tri_t*)malloc(sizeof(tri_t) * (size_t)g->nt);
    for (int64_t t = 0; t < g->nt; ++t) make_tri(g, t, &tris[t]);
    v2t_t a;
    build_v2t(g, &a);
    const int64_t N = g->N;
    memset(out, 0, sizeof(double) * (size_t)(np * N));
    double* ferg = (double*)calloc((size_t)(3 * np * g->nv), sizeof(double)); /* (3*np) x nv col-major */
    for (int m = 0; m < g->nmesh; ++m) {
        const double coeff = OO_MAGFACTOR * jump[m];
        for (int64_t i = 0; i < np; ++i) {
            v3 x = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
            #pragma omp parallel for schedule(static)
            for (int64_t v = g->mesh_vbeg[m]; v < g->mesh_vbeg[m + 1]; ++v) {
                v3 res = {0, 0, 0};
                for (int64_t k = a.beg[v]; k < a.beg[v + 1]; ++k) {
                    int64_t t = a.tri[k];
                    if (t < g->mesh_tbeg[m] || t >= g->mesh_tbeg[m + 1]) continue;
                    const tri_t* T = &tris[t];
                    int li = local_index(g, t, v);
                    static const int IDX[3][2] = {{1, 2}, {2, 0}, {0, 1}};
                    v3 A = T->p[IDX[li][0]], B = T->p[IDX[li][1]];
                    opS_t S;
                    opS_make(&S, T);
                    res = vadd(res, vscale(vsub(B, A), opS_eval(&S, x) / (2 * T->area)));
                }
                int64_t col = g->vidx[v];
                ferg[(size_t)col * 3 * np + 3 * i + 0] += res.x * coeff;
                ferg[(size_t)col * 3 * np + 3 * i + 1] += res.y * coeff;
                ferg[(size_t)col * 3 * np + 3 * i + 2] += res.z * coeff;
            }
        }
    }
    for (int64_t i = 0; i < np; ++i) {
        v3 dir = {ori[3 * i], ori[3 * i + 1], ori[3 * i + 2]};
        double dn = vnorm(dir);
        for (int64_t v = 0; v < g->nv; ++v) {
            int64_t col = g->vidx[v];
            v3 f = {ferg[(size_t)col * 3 * np + 3 * i], ferg[(size_t)col * 3 * np + 3 * i + 1],
                    ferg[(size_t)col * 3 * np + 3 * i + 2]};
            out[(size_t)col * np + i] = vdot(f, dir) / dn;
        }
    }
    free(ferg);
    free_v2t(&a);
    free(tris);
    return 0;
}

/* DipSource2MEGMat (assembleSensors.cpp:133-159): nsens x ndip col-major. */
int oo_ds2mm(const double* dip, int64_t ndip, const double* pos, const double* ori, int64_t np, double* out) {
    for (int64_t i = 0; i < np; ++i)
        for (int64_t j = 0; j < ndip; ++j) {
            v3 r = {dip[6 * j], dip[6 * j + 1], dip[6 * j + 2]};
            v3 q = {dip[6 * j + 3], dip[6 * j + 4], dip[6 * j + 5]};
            v3 diff = vsub((v3){pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]}, r);
            double nd = vnorm(diff);
            v3 f = vscale(vcross(q, diff), 1.0 / (nd * nd * nd));
            v3 dir = {ori[3 * i], ori[3 * i + 1], ori[3 * i + 2]};
            out[(size_t)j * np + i] = vdot(f, dir) * OO_MAGFACTOR / vnorm(dir);
        }
    return 0;
}

int oo_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oo_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
