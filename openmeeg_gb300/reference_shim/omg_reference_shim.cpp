// OpenMEEG's own C++ API on the GB300 library: a drop-in shared library that
// defines the forward-path functions of the reference (same names, same
// signatures, same return types) on top of the C ABI of libomg_gb300.so.
//
// Programs written against OpenMEEG -- including the reference's unmodified
// om_assemble and om_gain -- are linked with this library ahead of the
// reference library (link order, or LD_PRELOAD); the dynamic linker then
// binds their calls, and the reference library's own internal calls, to the
// definitions below:
//
//   SymMatrix HeadMat(const Geometry&, const Integrator&)        assembleHeadMat.cpp:133-135
//   Matrix SourceMatrix<Dipole>(geo, dipoles, integrator, domain) assembleSourceMat.cpp:66-104
//   SparseMatrix Head2EEGMat(const Geometry&, const Sensors&)     assembleSensors.cpp:25-39
//   Matrix Head2MEGMat(const Geometry&, const Sensors&)           assembleSensors.cpp:69-96
//   Matrix DipSource2MEGMat(const Matrix&, const Sensors&)        assembleSensors.cpp:133-159
//   Matrix SymMatrix::solveLin(Matrix&) const                     symmatrix.cpp:133-152
//
// GainEEGadjoint / GainMEGadjoint / GainEEGMEGadjoint (gain.h:78-136) are
// inline in the reference's header and call SymMatrix::solveLin and
// SourceMatrix<Dipole>, so they run on the GPU through these two.
//
// The library needs the geometry files: the shim also wraps
// Geometry::read_geometry_file / read_conductivity_file (geometry.cpp:180,231)
// to note, per Geometry object, the files it was read from (the reference's
// code runs unchanged; the wrapper calls it through dlsym(RTLD_NEXT)).  A call
// the library does not cover -- a geometry built in memory, the old unknown
// ordering, sensors with several integration points or weights, a matrix
// solveLin cannot tie to a geometry read through this process -- goes to the
// reference's own implementation.  When the GPU library itself fails (no
// CUDA device, an error from the device), the shim throws (the drop-in fails
// loudly) unless OMG_SHIM_CPU_FALLBACK=1, which hands the call to the
// reference's implementation instead.
//
// Build (against a reference source tree and the reference library built from
// it): openmeeg_gb300/reference_shim/Makefile.
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <assemble.h>
#include <assembleSourceMat.h>
#include <dipole.h>
#include <geometry.h>
#include <integrator.h>
#include <matrix.h>
#include <sensors.h>
#include <sparse_matrix.h>
#include <symmatrix.h>

#include "openmeeg_gb300.h"

namespace {

using namespace OpenMEEG;

// ---- the library side: one context per process, device buffers per call
struct Dev {
    void* p = nullptr;
    explicit Dev(size_t bytes);
    ~Dev();
    Dev(const Dev&) = delete;
    Dev& operator=(const Dev&) = delete;
};

// Failures of the GPU library, raised as the reference's own exception type
// (OMExceptions.H) so callers handle them as they handle the reference's.
struct LibError : OpenMEEG::Exception {
    explicit LibError(const std::string& w) : OpenMEEG::Exception(w) {}
    OpenMEEG::ExceptionCode code() const noexcept override { return OpenMEEG::UNEXPECTED; }
};

// Device buffers of the shim's own copies (the CUDA runtime's primary context
// is the one the library works in, so the pointers are valid there).
Dev::Dev(size_t bytes) {
    if (bytes && cudaMalloc(&p, bytes) != cudaSuccess) throw LibError("openmeeg_gb300 shim: cudaMalloc failed");
}
Dev::~Dev() {
    if (p) cudaFree(p);
}
void h2d(void* d, const void* h, size_t n) {
    if (n && cudaMemcpy(d, h, n, cudaMemcpyHostToDevice) != cudaSuccess)
        throw LibError("openmeeg_gb300 shim: host-to-device copy failed");
}
void d2h(void* h, const void* d, size_t n) {
    if (n && cudaMemcpy(h, d, n, cudaMemcpyDeviceToHost) != cudaSuccess)
        throw LibError("openmeeg_gb300 shim: device-to-host copy failed");
}

void check(int rc, const char* what) {
    if (rc != OMG_OK) throw LibError(std::string("openmeeg_gb300 ") + what + ": " + omg_last_error());
}

bool cpu_fallback_allowed() {
    const char* e = std::getenv("OMG_SHIM_CPU_FALLBACK");
    return e && std::strcmp(e, "1") == 0;
}

std::mutex g_mutex;
omg_context g_ctx = nullptr;

omg_context context() {
    if (!g_ctx) check(omg_context_create(0, &g_ctx), "context");
    return g_ctx;
}

// Geometry objects read from files in this process: their files, and the
// library geometry made from them on first use.
struct GeoEntry {
    std::string geom, cond;
    omg_geometry handle = nullptr;
    int64_t N = -1;
};
std::map<const Geometry*, GeoEntry> g_geos;
const Geometry* g_last_geo = nullptr;

// The registry entry of `geo` when the library can take it (read from files
// here, numbered in the current ordering), else nullptr.  e->N is the head
// matrix dimension (nb_parameters minus the current-barrier triangles).
GeoEntry* library_geometry(const Geometry& geo) {
    auto it = g_geos.find(&geo);
    if (it == g_geos.end() || it->second.cond.empty()) return nullptr;
    GeoEntry& e = it->second;
    // the reference numbering of the library: all vertices first, then the triangles (the old ordering
    // interleaves them mesh by mesh)
    const size_t nv = geo.vertices().size();
    size_t barrier_triangles = 0;
    for (const auto& m : geo.meshes()) {
        if (m.current_barrier()) barrier_triangles += m.triangles().size();
        for (const auto& t : m.triangles())
            if (t.index() < nv && !m.current_barrier()) return nullptr;
    }
    e.N = (int64_t)(geo.nb_parameters() - barrier_triangles);
    return &e;
}

// The library's geometry of a registry entry (made from the files on first use).
omg_geometry handle(GeoEntry& e) {
    if (!e.handle) {
        check(omg_geometry_load(context(), e.geom.c_str(), e.cond.c_str(), &e.handle), "geometry");
        omg_geometry_info info;
        check(omg_geometry_get_info(e.handle, &info), "geometry info");
        if (info.n_unknowns != e.N) throw LibError("openmeeg_gb300 shim: the library numbers this geometry differently");
    }
    return e.handle;
}

// Integrator(order, levels, tol) fields (integrator.h:79-81; private, no
// accessors): read through a struct of the same layout, checked below.
struct IntegratorLayout {
    unsigned order;
    double tolerance;
    unsigned max_depth;
};
static_assert(sizeof(Integrator) == sizeof(IntegratorLayout), "Integrator layout changed: update the shim");

omg_integrator to_library(const Integrator& it) {
    IntegratorLayout l;
    std::memcpy(&l, &it, sizeof l);
    return omg_integrator{(int32_t)l.order, (int32_t)l.max_depth, l.tolerance};
}

// The reference's implementation of a function this library defines.
template <typename F>
F original(const char* mangled) {
    void* p = dlsym(RTLD_NEXT, mangled);
    if (!p) throw std::runtime_error(std::string("openmeeg_gb300 shim: reference symbol not found: ") + mangled);
    return reinterpret_cast<F>(p);
}

// Runs `gpu`; on a library failure, the reference's implementation when
// OMG_SHIM_CPU_FALLBACK=1, else the error.
template <typename R, typename G, typename C>
R gpu_or_reference(G gpu, C cpu) {
    try {
        return gpu();
    } catch (const LibError&) {
        if (cpu_fallback_allowed()) return cpu();
        throw;
    }
}

bool point_sensors(const Sensors& s) {
    if (s.getNumberOfPositions() != s.getNumberOfSensors()) return false;
    const Vector w = s.getWeights();
    for (size_t i = 0; i < w.nlin(); ++i)
        if (w(i) != 1.0) return false;
    return true;
}

// Row-major n x c host array of a column-major reference Matrix's first c columns.
std::vector<double> rows(const Matrix& M, size_t c) {
    std::vector<double> out(M.nlin() * c);
    for (size_t i = 0; i < M.nlin(); ++i)
        for (size_t j = 0; j < c; ++j) out[i * c + j] = M(i, j);
    return out;
}

std::vector<double> squids_of(const Sensors& s) {
    const Matrix& P = s.getPositions();
    const Matrix& O = s.getOrientations();
    std::vector<double> out(P.nlin() * 6);
    for (size_t i = 0; i < P.nlin(); ++i)
        for (int j = 0; j < 3; ++j) {
            out[i * 6 + j] = P(i, j);
            out[i * 6 + 3 + j] = O(i, j);
        }
    return out;
}

}  // namespace

namespace OpenMEEG {

// ---- geometry files ---------------------------------------------------------
void Geometry::read_geometry_file(const std::string& filename) {
    using F = void (*)(Geometry*, const std::string&);
    static F f = original<F>("_ZN8OpenMEEG8Geometry18read_geometry_fileERKNSt7__cxx1112basic_stringIcSt11char_traitsIcESaIcEEE");
    f(this, filename);
    std::lock_guard<std::mutex> lock(g_mutex);
    GeoEntry& e = g_geos[this];
    if (e.handle) omg_geometry_destroy(e.handle);
    e = GeoEntry{filename, "", nullptr, -1};
    g_last_geo = this;
}

void Geometry::read_conductivity_file(const std::string& filename) {
    using F = void (*)(Geometry*, const std::string&);
    static F f =
        original<F>("_ZN8OpenMEEG8Geometry22read_conductivity_fileERKNSt7__cxx1112basic_stringIcSt11char_traitsIcESaIcEEE");
    f(this, filename);
    std::lock_guard<std::mutex> lock(g_mutex);
    g_geos[this].cond = filename;
}

// ---- HeadMat ---------------------------------------------------------------
SymMatrix HeadMat(const Geometry& geo, const Integrator& integrator) {
    using F = SymMatrix (*)(const Geometry&, const Integrator&);
    static F ref = original<F>("_ZN8OpenMEEG7HeadMatERKNS_8GeometryERKNS_10IntegratorE");
    std::lock_guard<std::mutex> lock(g_mutex);
    GeoEntry* e = library_geometry(geo);
    if (!e) return ref(geo, integrator);
    return gpu_or_reference<SymMatrix>(
        [&] {
            const omg_geometry g = handle(*e);
            const omg_integrator it = to_library(integrator);
            const size_t n = (size_t)e->N, packed = n * (n + 1) / 2;
            Dev d(packed * sizeof(double));
            check(omg_headmat_packed_dev(context(), g, &it, static_cast<double*>(d.p)), "HeadMat");
            SymMatrix M(n);   // packed upper, i + j (j + 1) / 2 (symmatrix.h:55): the library's layout
            d2h(M.data(), d.p, packed * sizeof(double));
            return M;
        },
        [&] { return ref(geo, integrator); });
}

// ---- DipSourceMat ----------------------------------------------------------
template <>
Matrix SourceMatrix<Dipole>(const Geometry& geo, const Matrix& dipoles, const Integrator& integrator,
                            const std::string& domain_name) {
    using F = Matrix (*)(const Geometry&, const Matrix&, const Integrator&, const std::string&);
    static F ref = original<F>(
        "_ZN8OpenMEEG12SourceMatrixINS_6DipoleEEENS_6MatrixERKNS_8GeometryERKS2_RKNS_10IntegratorERKNSt7__cxx1112basic_"
        "stringIcSt11char_traitsIcESaIcEEE");
    std::lock_guard<std::mutex> lock(g_mutex);
    GeoEntry* e = library_geometry(geo);
    if (!e || dipoles.ncol() < 6) return ref(geo, dipoles, integrator, domain_name);
    int32_t domain = -1;
    if (!domain_name.empty()) {
        int32_t k = 0;
        for (const auto& d : geo.domains()) {
            if (d.name() == domain_name) domain = k;
            ++k;
        }
        if (domain < 0) return ref(geo, dipoles, integrator, domain_name);   // the reference reports it
    }
    return gpu_or_reference<Matrix>(
        [&] {
            const omg_geometry g = handle(*e);
            const omg_integrator it = to_library(integrator);
            const size_t nd = dipoles.nlin(), n = (size_t)e->N;
            const std::vector<double> dip = rows(dipoles, 6);
            Dev dd(dip.size() * sizeof(double)), out(n * nd * sizeof(double));
            h2d(dd.p, dip.data(), dip.size() * sizeof(double));
            check(omg_dipsourcemat_dev(context(), g, static_cast<double*>(dd.p), (int64_t)nd, &it, domain,
                                       static_cast<double*>(out.p)),
                  "DipSourceMat");
            Matrix M(n, nd);   // column-major, as the library writes it
            d2h(M.data(), out.p, n * nd * sizeof(double));
            return M;
        },
        [&] { return ref(geo, dipoles, integrator, domain_name); });
}

// ---- sensor matrices ---------------------------------------------------------
SparseMatrix Head2EEGMat(const Geometry& geo, const Sensors& electrodes) {
    using F = SparseMatrix (*)(const Geometry&, const Sensors&);
    static F ref = original<F>("_ZN8OpenMEEG11Head2EEGMatERKNS_8GeometryERKNS_7SensorsE");
    std::lock_guard<std::mutex> lock(g_mutex);
    GeoEntry* e = library_geometry(geo);
    if (!e) return ref(geo, electrodes);
    return gpu_or_reference<SparseMatrix>(
        [&] {
            const omg_geometry g = handle(*e);
            const size_t ne = electrodes.getNumberOfPositions(), n = (size_t)e->N;
            const std::vector<double> pos = rows(electrodes.getPositions(), 3);
            Dev dp(pos.size() * sizeof(double)), dense(ne * n * sizeof(double)), cols(ne * 3 * sizeof(int64_t)),
                vals(ne * 3 * sizeof(double));
            h2d(dp.p, pos.data(), pos.size() * sizeof(double));
            check(omg_head2eegmat_dev(context(), g, static_cast<double*>(dp.p), (int64_t)ne,
                                      static_cast<double*>(dense.p), static_cast<int64_t*>(cols.p),
                                      static_cast<double*>(vals.p)),
                  "Head2EEGMat");
            std::vector<int64_t> c(ne * 3);
            std::vector<double> v(ne * 3);
            d2h(c.data(), cols.p, c.size() * sizeof(int64_t));
            d2h(v.data(), vals.p, v.size() * sizeof(double));
            SparseMatrix M(ne, n);
            for (size_t i = 0; i < ne; ++i)
                for (int k = 0; k < 3; ++k) M(i, (size_t)c[3 * i + k]) = v[3 * i + k];
            return M;
        },
        [&] { return ref(geo, electrodes); });
}

Matrix Head2MEGMat(const Geometry& geo, const Sensors& sensors) {
    using F = Matrix (*)(const Geometry&, const Sensors&);
    static F ref = original<F>("_ZN8OpenMEEG11Head2MEGMatERKNS_8GeometryERKNS_7SensorsE");
    std::lock_guard<std::mutex> lock(g_mutex);
    GeoEntry* e = library_geometry(geo);
    if (!e || !point_sensors(sensors)) return ref(geo, sensors);
    return gpu_or_reference<Matrix>(
        [&] {
            const omg_geometry g = handle(*e);
            const size_t ns = sensors.getNumberOfSensors(), n = (size_t)e->N;
            const std::vector<double> sq = squids_of(sensors);
            Dev ds(sq.size() * sizeof(double)), out(ns * n * sizeof(double));
            h2d(ds.p, sq.data(), sq.size() * sizeof(double));
            check(omg_head2megmat_dev(context(), g, static_cast<double*>(ds.p), (int64_t)ns,
                                      static_cast<double*>(out.p)),
                  "Head2MEGMat");
            Matrix M(ns, n);
            d2h(M.data(), out.p, ns * n * sizeof(double));
            return M;
        },
        [&] { return ref(geo, sensors); });
}

Matrix DipSource2MEGMat(const Matrix& dipoles, const Sensors& sensors) {
    using F = Matrix (*)(const Matrix&, const Sensors&);
    static F ref = original<F>("_ZN8OpenMEEG16DipSource2MEGMatERKNS_6MatrixERKNS_7SensorsE");
    if (!point_sensors(sensors) || dipoles.ncol() < 6) return ref(dipoles, sensors);
    std::lock_guard<std::mutex> lock(g_mutex);
    return gpu_or_reference<Matrix>(
        [&] {
            const omg_context c = context();
            const size_t ns = sensors.getNumberOfSensors(), nd = dipoles.nlin();
            const std::vector<double> sq = squids_of(sensors), dip = rows(dipoles, 6);
            Dev ds(sq.size() * sizeof(double)), dd(dip.size() * sizeof(double)), out(ns * nd * sizeof(double));
            h2d(ds.p, sq.data(), sq.size() * sizeof(double));
            h2d(dd.p, dip.data(), dip.size() * sizeof(double));
            check(omg_dipsource2megmat_dev(c, static_cast<double*>(dd.p), (int64_t)nd,
                                           static_cast<double*>(ds.p), (int64_t)ns, static_cast<double*>(out.p)),
                  "DipSource2MEGMat");
            Matrix M(ns, nd);
            d2h(M.data(), out.p, ns * nd * sizeof(double));
            return M;
        },
        [&] { return ref(dipoles, sensors); });
}

// ---- SymMatrix::solveLin ----------------------------------------------------
// The library factors a head matrix with its quasi-definite LDL^T, which needs
// the geometry's [vertices | triangles] structure: the matrix is tied to the
// most recent geometry read in this process whose unknown count it has and
// whose diagonal has that structure's signs (negative on the vertex unknowns,
// positive on the triangle unknowns); any other matrix goes to the reference's
// Bunch-Kaufman solve.
Matrix SymMatrix::solveLin(Matrix& RHS) const {
    using F = Matrix (*)(const SymMatrix*, Matrix&);
    static F ref = original<F>("_ZNK8OpenMEEG9SymMatrix8solveLinERNS_6MatrixE");
    std::lock_guard<std::mutex> lock(g_mutex);
    const size_t n = nlin();
    GeoEntry* e = nullptr;
    if (g_last_geo && g_geos.count(g_last_geo)) {
        e = library_geometry(*g_last_geo);
        if (e && (size_t)e->N != n) e = nullptr;
    }
    if (!e || RHS.nlin() != n) return ref(this, RHS);
    const size_t nv = g_last_geo->vertices().size();
    for (size_t i = 0; i < n; ++i) {
        const double d = (*this)(i, i);
        if (!((i < nv) ? d < 0.0 : d > 0.0)) return ref(this, RHS);
    }
    return gpu_or_reference<Matrix>(
        [&] {
            const omg_geometry g = handle(*e);
            std::vector<double> dense(n * n);
            for (size_t j = 0; j < n; ++j)
                for (size_t i = 0; i < n; ++i) dense[i + j * n] = (*this)(i, j);
            Dev dh(n * n * sizeof(double)), db(n * RHS.ncol() * sizeof(double));
            h2d(dh.p, dense.data(), n * n * sizeof(double));
            h2d(db.p, RHS.data(), n * RHS.ncol() * sizeof(double));
            omg_solver sv = nullptr;
            check(omg_solver_from_headmat_dev(context(), g, static_cast<double*>(dh.p), (int64_t)n,
                                              OMG_PREC_FP64, &sv),
                  "solveLin (factorization)");
            const int rc = omg_solver_solve_dev(sv, static_cast<double*>(db.p), (int64_t)n, (int64_t)RHS.ncol());
            omg_solver_destroy(sv);
            check(rc, "solveLin (solve)");
            d2h(RHS.data(), db.p, n * RHS.ncol() * sizeof(double));
            return RHS;
        },
        [&] { return ref(this, RHS); });
}

}  // namespace OpenMEEG
