// Host-side geometry bookkeeping: the GB300 library's restatement of what
// OpenMEEG's Geometry does before assembly.  Kept on the host: it is O(n)
// integer work done once per head model.
//
//   interface orientation   OpenMEEG/src/interface.cpp:55-95
//   domain/mesh orientation OpenMEEG/include/domain.h:43-45,95-101
//   current barriers        OpenMEEG/src/geometry.cpp:424-536
//   numbering               OpenMEEG/src/geometry.cpp:256-295
//   mesh pairs              OpenMEEG/src/geometry.cpp:405-420
//   pair coefficients       OpenMEEG/src/assembleHeadMat.cpp:92-95
//   nestedness              OpenMEEG/src/geometry.cpp:369-401
#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <fstream>
#include <future>
#include <map>
#include <set>
#include <sstream>

#include "omg_internal.h"

namespace omg {

namespace {

bool almost_equal(double x, double y, double eps = 1e3) {   // OpenMEEG/include/om_common.h:24-26
    return std::fabs(x - y) < DBL_EPSILON * std::fabs(x + y) * eps || std::fabs(x - y) < DBL_MIN;
}

// Triangle::solid_angle (OpenMEEG/include/triangle.h:123-136) summed over a mesh.
double mesh_solid_angle(const HostGeometry& g, int m, const double p[3]) {
    double total = 0.0;
    for (int64_t t = g.tbeg[m]; t < g.tbeg[m + 1]; ++t) {
        const double* a = &g.V[3 * (size_t)g.T[3 * t]];
        const double* b = &g.V[3 * (size_t)g.T[3 * t + 1]];
        const double* c = &g.V[3 * (size_t)g.T[3 * t + 2]];
        double r[3][3], d[3];
        for (int k = 0; k < 3; ++k) {
            r[0][k] = a[k] - p[k];
            r[1][k] = b[k] - p[k];
            r[2][k] = c[k] - p[k];
        }
        for (int i = 0; i < 3; ++i) d[i] = std::sqrt(r[i][0] * r[i][0] + r[i][1] * r[i][1] + r[i][2] * r[i][2]);
        double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        double nn[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        // twice the area times the signed height of p: r0 . (e1 x e2)
        const double dd = r[0][0] * nn[0] + r[0][1] * nn[1] + r[0][2] * nn[2];
        auto dot = [&](int i, int j) { return r[i][0] * r[j][0] + r[i][1] * r[j][1] + r[i][2] * r[j][2]; };
        double den = d[0] * d[1] * d[2] + (d[0] * dot(1, 2) + d[1] * dot(2, 0) + d[2] * dot(0, 1));
        total += (std::fabs(dd) < 1e-10) ? 0.0 : 2 * std::atan2(dd, den);
    }
    return total;
}

}  // namespace

int HostGeometry::mesh_orientation(int d, int m) const {   // domain.h:43-45, 95-101
    for (const auto& b : domains[d].bounds)
        if (b.mesh == m) return b.inside ? b.o : -b.o;
    return 0;
}

std::vector<int> HostGeometry::domains_of(int m) const {
    std::vector<int> r;
    for (int d = 0; d < (int)domains.size(); ++d)
        if (mesh_orientation(d, m) != 0) r.push_back(d);
    return r;
}

double HostGeometry::conductivity_jump(int m) const {   // geometry.h:188-194
    double res = 0.0;
    for (int d : domains_of(m)) res += domains[d].sigma * mesh_orientation(d, m);
    return res;
}

void HostGeometry::recompute_coefficients() {
    // make_mesh_pairs + coefficients; pairs keep their order.
    pairs.clear();
    for (int m1 = 0; m1 < nmesh; ++m1) {
        for (int m2 = 0; m2 <= m1; ++m2) {
            std::vector<int> d1 = domains_of(m1), d2 = domains_of(m2), common;
            std::set_intersection(d1.begin(), d1.end(), d2.begin(), d2.end(), std::back_inserter(common));
            int orientation;
            if (m1 == m2)
                orientation = 1;
            else
                orientation = common.empty()
                                  ? 0
                                  : (mesh_orientation(common[0], m1) == mesh_orientation(common[0], m2) ? 1 : -1);
            double sig = 0.0, sinv = 0.0;
            for (int d : common) {
                sig += domains[d].sigma;
                sinv += 1.0 / domains[d].sigma;   // +inf for a zero-conductivity domain, as in the reference
            }
            if (sig != 0.0 && orientation != 0) {
                const double factor = orientation * kK;
                pairs.push_back({m1, m2, orientation, factor * sinv, factor * sig, -factor * (double)common.size()});
            }
        }
    }
}

void HostGeometry::finalize() {
    nv = (int64_t)V.size() / 3;
    nt = (int64_t)T.size() / 3;
    // distinct vertices: copies with equal coordinates are one unknown (Geometry::add_vertex,
    // geometry.h:100-108), numbered in order of first appearance
    {
        // an open-addressing table over the coordinates' bit patterns (-0.0 folded into +0.0, so equal
        // coordinates hash equally; the coordinates are finite), probed linearly; each slot holds the first
        // vertex with its coordinates: the numbering of an ordered map in linear time, without allocations
        auto bits = [this](int64_t v, int c) {
            const double x = V[3 * v + c] + 0.0;   // -0.0 + 0.0 = +0.0
            uint64_t b;
            std::memcpy(&b, &x, sizeof b);
            return b;
        };
        size_t cap = 16;
        while (cap < 2 * (size_t)nv) cap <<= 1;
        std::vector<int64_t> slot(cap, -1);
        vglob.assign(nv, 0);
        int64_t count = 0;
        for (int64_t v = 0; v < nv; ++v) {
            uint64_t h = 0x9E3779B97F4A7C15ull;
            for (int c = 0; c < 3; ++c) {
                h ^= bits(v, c) + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
                h *= 0xBF58476D1CE4E5B9ull;
            }
            size_t i = (size_t)(h ^ (h >> 31)) & (cap - 1);
            for (;; i = (i + 1) & (cap - 1)) {
                const int64_t u = slot[i];
                if (u < 0) {
                    slot[i] = v;
                    vglob[v] = count++;
                    break;
                }
                if (V[3 * u] == V[3 * v] && V[3 * u + 1] == V[3 * v + 1] && V[3 * u + 2] == V[3 * v + 2]) {
                    vglob[v] = vglob[u];
                    break;
                }
            }
        }
        nvg = count;
        shared = nvg < nv;
    }
    // Interface orientation (interface.cpp:55-95): the solid angle at the bounding-box centre of the
    // interface, summed over its oriented meshes, must be -4 pi or 0; +4 pi flips the interface.
    // the interfaces' sums are independent: one thread each on large geometries (each sum in mesh order)
    auto iface_angle = [this](size_t i) {
        double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
        for (const auto& om : ifaces[i])
            for (int64_t v = vbeg[om.first]; v < vbeg[om.first + 1]; ++v)
                for (int k = 0; k < 3; ++k) {
                    lo[k] = std::min(lo[k], V[3 * v + k]);
                    hi[k] = std::max(hi[k], V[3 * v + k]);
                }
        const double c[3] = {0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1]), 0.5 * (lo[2] + hi[2])};
        double s = 0.0;
        for (const auto& om : ifaces[i]) s += om.second * mesh_solid_angle(*this, om.first, c);
        return s;
    };
    std::vector<double> angle(ifaces.size(), 0.0);
    if (ifaces.size() > 1 && nt >= 8192) {
        std::vector<std::future<double>> fut;
        for (size_t i = 1; i < ifaces.size(); ++i) fut.push_back(std::async(std::launch::async, iface_angle, i));
        angle[0] = iface_angle(0);
        for (size_t i = 1; i < ifaces.size(); ++i) angle[i] = fut[i - 1].get();
    } else {
        for (size_t i = 0; i < ifaces.size(); ++i) angle[i] = iface_angle(i);
    }
    for (size_t i = 0; i < ifaces.size(); ++i) {
        double s = angle[i];
        if (almost_equal(s, 4 * M_PI)) {
            for (auto& om : ifaces[i]) om.second = -om.second;
            s = -s;
        }
        if (!(almost_equal(s, 0.0) || almost_equal(s, -4 * M_PI)))
            throw Error(OMG_ERR_INVALID, "interface " + std::to_string(i + 1) +
                                             " is not closed or its bounding-box centre lies outside it");
    }
    // domain boundaries, mesh by mesh
    orient.assign(nmesh, 0);
    for (auto& d : domains) {
        d.bounds.clear();
        for (size_t k = 0; k < d.ifb.size(); ++k)
            for (const auto& om : ifaces[d.ifb[k].iface])
                d.bounds.push_back({om.first, d.ifb[k].inside, om.second, (int)k});
    }
    for (const auto& itf : ifaces)
        for (const auto& om : itf)
            if (orient[om.first] == 0) orient[om.first] = om.second;
    for (int m = 0; m < nmesh; ++m)
        if (orient[m] == 0) orient[m] = 1;
    // mark_current_barriers (geometry.cpp:424-536)
    barrier.assign(nmesh, 0);
    outermost.assign(nmesh, 0);
    std::vector<int> isolated(nmesh, 0);
    for (const auto& d : domains)
        if (almost_equal(d.sigma, 0.0))
            for (const auto& b : d.bounds) {
                if (barrier[b.mesh]) {
                    isolated[b.mesh] = 1;
                    outermost[b.mesh] = 0;
                }
                barrier[b.mesh] = 1;
            }
    for (const auto& d : domains)
        if (almost_equal(d.sigma, 0.0))
            for (const auto& b : d.bounds)
                if (!b.inside && barrier[b.mesh] && !isolated[b.mesh]) outermost[b.mesh] = 1;
    for (int m = 0; m < nmesh; ++m)
        if (isolated[m])
            throw Error(OMG_ERR_UNSUPPORTED, "meshes touching non-conductive domains on both sides are not supported");
    // independent parts: BFS over meshes sharing a domain, candidates in mesh order
    std::vector<int> cand(nmesh);
    for (int m = 0; m < nmesh; ++m) cand[m] = m;
    std::vector<std::vector<int>> parts;
    while (!cand.empty()) {
        int c0 = cand.front();
        cand.erase(cand.begin());
        std::vector<int> conn{c0}, pend{c0};
        while (!pend.empty()) {
            int cur = pend.front();
            pend.erase(pend.begin());
            std::vector<int> keep;
            std::vector<int> dc = domains_of(cur);
            for (int it : cand) {
                std::vector<int> di = domains_of(it), common;
                std::set_intersection(dc.begin(), dc.end(), di.begin(), di.end(), std::back_inserter(common));
                if (common.empty())
                    keep.push_back(it);
                else {
                    conn.push_back(it);
                    pend.push_back(it);
                }
            }
            cand = keep;
        }
        if (conn.size() > 1 || !isolated[conn[0]]) parts.push_back(conn);
    }
    // outermost domain (geometry.cpp:23-41) -> its meshes are outermost
    for (const auto& d : domains) {
        bool outer = true;
        for (const auto& b : d.bounds)
            if (b.inside) outer = false;
        if (outer) {
            for (const auto& b : d.bounds) outermost[b.mesh] = 1;
            break;
        }
    }
    // nestedness (geometry.cpp:369-401), first criterion
    nested = true;
    for (const auto& d : domains) {
        bool outer = true;
        for (const auto& b : d.bounds)
            if (b.inside) outer = false;
        if (outer) continue;
        int n_in = 0;
        for (const auto& b : d.ifb)
            if (b.inside) ++n_in;
        if (n_in >= 2) nested = false;
    }
    // numbering (geometry.cpp:256-295)
    tidx.assign(nt, -1);
    int64_t idx = nvg;
    for (int m = 0; m < nmesh; ++m)
        if (!barrier[m])
            for (int64_t t = tbeg[m]; t < tbeg[m + 1]; ++t) tidx[t] = idx++;
    nP = idx - nvg;
    int64_t nbar = 0;
    for (int m = 0; m < nmesh; ++m)
        if (barrier[m]) {
            nbar += tbeg[m + 1] - tbeg[m];
            for (int64_t t = tbeg[m]; t < tbeg[m + 1]; ++t) tidx[t] = idx++;
        }
    N = idx - nbar;
    recompute_coefficients();
    part_outermost.clear();
    for (const auto& part : parts) {
        std::vector<int> om;
        for (int m : part)
            if (outermost[m]) om.push_back(m);
        part_outermost.push_back(om);
    }
    eeg_ifaces.clear();   // dist_point_geom (danielsson.cpp:107-128): boundaries of zero-conductivity domains
    for (const auto& d : domains)
        if (d.sigma == 0.0)
            for (const auto& b : d.ifb) eeg_ifaces.push_back(b.iface);
    // vertex -> triangle adjacency
    v2t_beg.assign(nv + 1, 0);
    for (int64_t t = 0; t < nt; ++t)
        for (int j = 0; j < 3; ++j) v2t_beg[T[3 * t + j] + 1]++;
    for (int64_t v = 0; v < nv; ++v) v2t_beg[v + 1] += v2t_beg[v];
    v2t_tri.assign(v2t_beg[nv], 0);
    v2t_loc.assign(v2t_beg[nv], 0);
    std::vector<int32_t> fill(nv, 0);
    for (int64_t t = 0; t < nt; ++t)
        for (int j = 0; j < 3; ++j) {
            int32_t v = T[3 * t + j];
            v2t_tri[v2t_beg[v] + fill[v]] = (int32_t)t;
            v2t_loc[v2t_beg[v] + fill[v]] = (int8_t)j;
            fill[v]++;
        }
}

static HostGeometry build_geometry_impl(int nmesh, const int64_t* nverts, const double* verts, const int64_t* ntris,
                                       const int64_t* tris, const std::vector<std::vector<std::pair<int, int>>>& ifaces,
                                       int ndom, const int32_t* nb, const int32_t* bounds, const double* sigma,
                                       const std::vector<std::string>& dom_names);

// Meshes given as interfaces (one mesh each, normal orientation).
HostGeometry build_geometry(int nmesh, const int64_t* nverts, const double* verts, const int64_t* ntris,
                            const int64_t* tris, int ndom, const int32_t* nb, const int32_t* bounds,
                            const double* sigma, const std::vector<std::string>& dom_names) {
    std::vector<std::vector<std::pair<int, int>>> ifaces;
    for (int m = 0; m < nmesh; ++m) ifaces.push_back({{m, 1}});
    return build_geometry_impl(nmesh, nverts, verts, ntris, tris, ifaces, ndom, nb, bounds, sigma, dom_names);
}

static HostGeometry build_geometry_impl(int nmesh, const int64_t* nverts, const double* verts, const int64_t* ntris,
                                       const int64_t* tris, const std::vector<std::vector<std::pair<int, int>>>& ifaces,
                                       int ndom, const int32_t* nb, const int32_t* bounds, const double* sigma,
                                       const std::vector<std::string>& dom_names) {
    OMG_REQUIRE(nmesh > 0 && ndom > 0, "geometry needs at least one mesh and one domain");
    HostGeometry g;
    g.nmesh = nmesh;
    g.ifaces = ifaces;
    g.vbeg.assign(nmesh + 1, 0);
    g.tbeg.assign(nmesh + 1, 0);
    for (int m = 0; m < nmesh; ++m) {
        OMG_REQUIRE(nverts[m] >= 3 && ntris[m] >= 1, "empty mesh");
        g.vbeg[m + 1] = g.vbeg[m] + nverts[m];
        g.tbeg[m + 1] = g.tbeg[m] + ntris[m];
    }
    OMG_REQUIRE(g.vbeg[nmesh] < (int64_t)INT32_MAX && g.tbeg[nmesh] < (int64_t)INT32_MAX, "mesh too large");
    g.V.assign(verts, verts + 3 * g.vbeg[nmesh]);
    for (double x : g.V) OMG_REQUIRE(std::isfinite(x), "non-finite vertex coordinate");
    g.T.resize(3 * g.tbeg[nmesh]);
    for (int m = 0; m < nmesh; ++m)
        for (int64_t t = g.tbeg[m]; t < g.tbeg[m + 1]; ++t)
            for (int j = 0; j < 3; ++j) {
                int64_t lv = tris[3 * t + j];
                OMG_REQUIRE(lv >= 0 && lv < nverts[m], "triangle vertex index out of range");
                g.T[3 * t + j] = (int32_t)(g.vbeg[m] + lv);
            }
    // degenerate triangles make the analytic kernels divide by zero
    for (int64_t t = 0; t < g.tbeg[nmesh]; ++t) {
        const double* a = &g.V[3 * (size_t)g.T[3 * t]];
        const double* b = &g.V[3 * (size_t)g.T[3 * t + 1]];
        const double* c = &g.V[3 * (size_t)g.T[3 * t + 2]];
        double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        double nn[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        OMG_REQUIRE(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2] > 0.0,
                    "degenerate (zero-area) triangle " + std::to_string(t));
    }
    int k = 0;
    for (int d = 0; d < ndom; ++d) {
        Domain dom;
        dom.name = d < (int)dom_names.size() ? dom_names[d] : ("domain" + std::to_string(d));
        OMG_REQUIRE(std::isfinite(sigma[d]) && sigma[d] >= 0.0, "conductivity must be finite and >= 0");
        dom.sigma = sigma[d];
        for (int j = 0; j < nb[d]; ++j, ++k) {
            int b = bounds[k];
            OMG_REQUIRE(b != 0 && std::abs(b) <= (int)g.ifaces.size(), "domain boundary refers to an unknown interface");
            dom.ifb.push_back({std::abs(b) - 1, b < 0});   // GeomFile.h:289-291
        }
        g.domains.push_back(dom);
    }
    g.finalize();
    return g;
}

HostGeometry build_geometry_interfaces(int nmesh, const int64_t* nverts, const double* verts, const int64_t* ntris,
                                       const int64_t* tris, int nif, const int32_t* if_nm, const int32_t* if_meshes,
                                       int ndom, const int32_t* nb, const int32_t* bounds, const double* sigma,
                                       const std::vector<std::string>& dom_names) {
    OMG_REQUIRE(nif > 0, "geometry needs at least one interface");
    std::vector<std::vector<std::pair<int, int>>> ifaces(nif);
    int k = 0;
    for (int i = 0; i < nif; ++i) {
        OMG_REQUIRE(if_nm[i] > 0, "empty interface");
        for (int j = 0; j < if_nm[i]; ++j, ++k) {
            const int m = if_meshes[k];
            OMG_REQUIRE(m != 0 && std::abs(m) <= nmesh, "interface refers to an unknown mesh");
            ifaces[i].push_back({std::abs(m) - 1, m > 0 ? 1 : -1});
        }
    }
    return build_geometry_impl(nmesh, nverts, verts, ntris, tris, ifaces, ndom, nb, bounds, sigma, dom_names);
}

// ---- file loaders -----------------------------------------------------------

namespace {

std::string strip_comment(const std::string& s) {
    auto p = s.find('#');
    return p == std::string::npos ? s : s.substr(0, p);
}

void read_tri(const std::string& path, std::vector<double>& V, std::vector<int64_t>& T) {
    std::ifstream f(path);
    if (!f) throw Error(OMG_ERR_IO, "cannot open mesh " + path);
    char ch;
    int64_t nv;
    f >> ch >> nv;
    if (!f || nv <= 0) throw Error(OMG_ERR_IO, "bad .tri header in " + path);
    V.resize(3 * nv);
    for (int64_t i = 0; i < nv; ++i) {
        double n[3];
        f >> V[3 * i] >> V[3 * i + 1] >> V[3 * i + 2] >> n[0] >> n[1] >> n[2];
    }
    int64_t nt, nt2, nt3;
    f >> ch >> nt >> nt2 >> nt3;
    if (!f || nt <= 0) throw Error(OMG_ERR_IO, "bad .tri triangle header in " + path);
    T.resize(3 * nt);
    for (int64_t i = 0; i < 3 * nt; ++i) f >> T[i];
    if (!f) throw Error(OMG_ERR_IO, "truncated .tri file " + path);
}

}  // namespace

// .geom v1.1 (GeomFile.h:160-300): an optional "Meshes" section of named
// mesh files, "Interfaces" given either as mesh files (one mesh each) or as
// lists of +/-mesh names, and "Domains" as lists of +/-interface names (a '-'
// means inside, '+' or no sign outside; "shared" ends the list).  Entries
// without a "Name:" get the names "1", "2", ... in order.  Meshes are .tri or
// .off files.  Vertices with equal coordinates in several meshes are one
// unknown (shared vertices).
namespace {

struct GeomEntry {
    std::string name, rest;   // rest: the line after "Keyword name:" (or the whole line)
};

GeomEntry split_entry(const std::string& line, const std::string& keyword, unsigned index) {
    std::string s = line;
    s.erase(0, s.find_first_not_of(" \t\r"));
    GeomEntry e;
    e.name = std::to_string(index + 1);
    if (s.compare(0, keyword.size(), keyword) == 0) {
        std::string after = s.substr(keyword.size());
        auto c = after.find(':');
        if (c != std::string::npos) {
            std::string nm = after.substr(0, c);
            nm.erase(0, nm.find_first_not_of(" \t"));
            nm.erase(nm.find_last_not_of(" \t\r") == std::string::npos ? 0 : nm.find_last_not_of(" \t\r") + 1);
            if (!nm.empty()) e.name = nm;
            e.rest = after.substr(c + 1);
            return e;
        }
    }
    e.rest = s;
    return e;
}

std::string entry_filename(const std::string& rest, const std::string& dir) {
    std::string fn;
    auto q1 = rest.find('"');
    if (q1 != std::string::npos) {
        fn = rest.substr(q1 + 1, rest.find('"', q1 + 1) - q1 - 1);
    } else {
        std::istringstream es(rest);
        es >> fn;
    }
    if (fn.empty()) throw Error(OMG_ERR_IO, "missing file name in geometry file");
    return fn[0] == '/' ? fn : dir + fn;
}

std::vector<std::string> tokens_of(const std::string& s) {
    std::istringstream is(s);
    std::vector<std::string> out;
    std::string t;
    while (is >> t) out.push_back(t);
    return out;
}

// OFF (MeshIOs/off.h): "OFF", "nv nt 0", nv vertices, nt lines "3 i j k".
void read_off(const std::string& path, std::vector<double>& V, std::vector<int64_t>& T) {
    std::ifstream f(path);
    if (!f) throw Error(OMG_ERR_IO, "cannot open mesh " + path);
    std::string magic;
    f >> magic;
    if (magic != "OFF") throw Error(OMG_ERR_IO, "not an OFF file: " + path);
    std::string tok;
    int64_t nv = 0, nt = 0, ne = 0;
    while (f >> tok && tok[0] == '#') std::getline(f, tok);   // comments before the counts
    nv = std::stoll(tok);
    f >> nt >> ne;
    if (!f || nv <= 0 || nt <= 0) throw Error(OMG_ERR_IO, "bad OFF header in " + path);
    V.resize(3 * nv);
    for (int64_t i = 0; i < 3 * nv; ++i) f >> V[i];
    T.resize(3 * nt);
    for (int64_t i = 0; i < nt; ++i) {
        int64_t k;
        f >> k >> T[3 * i] >> T[3 * i + 1] >> T[3 * i + 2];
        if (k != 3) throw Error(OMG_ERR_UNSUPPORTED, "OFF faces must be triangles: " + path);
    }
    if (!f) throw Error(OMG_ERR_IO, "truncated OFF file " + path);
}

void read_mesh_file(const std::string& path, std::vector<double>& V, std::vector<int64_t>& T) {
    const auto dot = path.find_last_of('.');
    const std::string ext = dot == std::string::npos ? "" : path.substr(dot + 1);
    if (ext == "tri")
        read_tri(path, V, T);
    else if (ext == "off")
        read_off(path, V, T);
    else
        throw Error(OMG_ERR_UNSUPPORTED, "mesh format not supported (only .tri and .off): " + path);
}

}  // namespace

HostGeometry load_geometry_files(const std::string& geom, const std::string& cond) {
    std::ifstream f(geom);
    if (!f) throw Error(OMG_ERR_IO, "cannot open geometry file " + geom);
    std::string line;
    std::getline(f, line);
    if (line.find("# Domain Description 1.1") == std::string::npos)
        throw Error(OMG_ERR_UNSUPPORTED, "only '# Domain Description 1.1' geometry files are supported");
    std::string dir = geom.substr(0, geom.find_last_of('/') == std::string::npos ? 0 : geom.find_last_of('/') + 1);
    std::vector<std::string> lines;
    while (std::getline(f, line)) {
        std::string s = strip_comment(line);
        if (s.find_first_not_of(" \t\r") != std::string::npos) lines.push_back(s);
    }
    std::vector<std::string> mesh_names, mesh_files;
    std::vector<std::string> iface_names;
    std::vector<std::vector<std::pair<std::string, bool>>> iface_meshes;   // (mesh name, normal orientation)
    std::vector<std::string> dnames;
    std::vector<std::vector<std::pair<std::string, bool>>> dbounds;        // (interface name, inside)
    bool mesh_section = false;
    for (size_t i = 0; i < lines.size(); ++i) {
        std::vector<std::string> head = tokens_of(lines[i]);
        const std::string& key = head[0];
        if (key == "MeshFile") {
            throw Error(OMG_ERR_UNSUPPORTED, "geometry given as one mesh file (MeshFile) is not supported");
        } else if (key == "Meshes") {
            mesh_section = true;
            const int n = std::stoi(head.at(1));
            for (int k = 0; k < n; ++k) {
                GeomEntry e = split_entry(lines.at(++i), "Mesh", (unsigned)k);
                mesh_names.push_back(e.name);
                mesh_files.push_back(entry_filename(e.rest, dir));
            }
        } else if (key == "Interfaces") {
            const int n = std::stoi(head.at(1));
            for (int k = 0; k < n; ++k) {
                GeomEntry e = split_entry(lines.at(++i), "Interface", (unsigned)k);
                iface_names.push_back(e.name);
                if (!mesh_section) {   // meshes given as interfaces
                    mesh_names.push_back(e.name);
                    mesh_files.push_back(entry_filename(e.rest, dir));
                    iface_meshes.push_back({{e.name, true}});
                } else {
                    std::vector<std::pair<std::string, bool>> om;
                    for (std::string t : tokens_of(e.rest)) {
                        bool normal = true;
                        if (t[0] == '+' || t[0] == '-') {
                            normal = t[0] == '+';
                            t = t.substr(1);
                        }
                        om.push_back({t, normal});
                    }
                    iface_meshes.push_back(om);
                }
            }
        } else if (key == "Domains") {
            const int n = std::stoi(head.at(1));
            for (int k = 0; k < n; ++k) {
                GeomEntry e = split_entry(lines.at(++i), "Domain", (unsigned)k);
                std::vector<std::pair<std::string, bool>> b;
                for (std::string t : tokens_of(e.rest)) {
                    if (t == "shared") break;
                    bool inside = false;
                    if (t[0] == '+' || t[0] == '-') {
                        inside = t[0] == '-';
                        t = t.substr(1);
                    }
                    b.push_back({t, inside});
                }
                dnames.push_back(e.name);
                dbounds.push_back(b);
            }
        }
    }
    if (mesh_files.empty() || dnames.empty()) throw Error(OMG_ERR_IO, "no interfaces or domains in " + geom);
    auto find = [](const std::vector<std::string>& v, const std::string& x) {
        return (int)(std::find(v.begin(), v.end(), x) - v.begin());
    };
    std::vector<int32_t> if_nm, if_meshes;
    for (size_t k = 0; k < iface_names.size(); ++k) {
        if_nm.push_back((int32_t)iface_meshes[k].size());
        for (const auto& om : iface_meshes[k]) {
            const int m = find(mesh_names, om.first);
            if (m == (int)mesh_names.size()) throw Error(OMG_ERR_INVALID, "unknown mesh " + om.first);
            if_meshes.push_back(om.second ? m + 1 : -(m + 1));
        }
    }
    std::vector<int32_t> nb, bounds;
    for (size_t d = 0; d < dnames.size(); ++d) {
        for (const auto& b : dbounds[d]) {
            const int k = find(iface_names, b.first);
            if (k == (int)iface_names.size())
                throw Error(OMG_ERR_INVALID, "domain " + dnames[d] + " refers to an unknown interface " + b.first);
            bounds.push_back(b.second ? -(k + 1) : (k + 1));
        }
        nb.push_back((int32_t)dbounds[d].size());
    }
    std::map<std::string, double> sig;
    std::ifstream fc(cond);
    if (!fc) throw Error(OMG_ERR_IO, "cannot open conductivity file " + cond);
    while (std::getline(fc, line)) {
        std::istringstream is(strip_comment(line));
        std::string name;
        double v;
        if (is >> name >> v) sig[name] = v;
    }
    std::vector<double> sigma;
    for (const auto& n : dnames) {
        auto it = sig.find(n);
        if (it == sig.end()) throw Error(OMG_ERR_INVALID, "no conductivity for domain " + n);
        sigma.push_back(it->second);
    }
    std::vector<double> V;
    std::vector<int64_t> T, nv, nt;
    for (const auto& m : mesh_files) {
        std::vector<double> v;
        std::vector<int64_t> t;
        read_mesh_file(m, v, t);
        V.insert(V.end(), v.begin(), v.end());
        T.insert(T.end(), t.begin(), t.end());
        nv.push_back((int64_t)v.size() / 3);
        nt.push_back((int64_t)t.size() / 3);
    }
    return build_geometry_interfaces((int)mesh_files.size(), nv.data(), V.data(), nt.data(), T.data(),
                                     (int)iface_names.size(), if_nm.data(), if_meshes.data(), (int)dnames.size(),
                                     nb.data(), bounds.data(), sigma.data(), dnames);
}

}  // namespace omg

// Test hook (not part of the public header; host only, no device needed): the
// numbering a geometry loaded from .geom / .cond files gets.  sizes receives
// {meshes, vertex copies, distinct vertices, triangles, unknowns N, triangle
// unknowns}; when the capacities suffice, V (copies x 3), vglob (copy ->
// distinct vertex), tidx (triangle -> unknown, reference order), orient and
// barrier (per mesh) are filled too.  Returns 0, or -1 with nothing written
// past sizes when the files are refused.
extern "C" int omg_internal_geometry_numbering(const char* geom, const char* cond, int64_t* sizes, double* V,
                                               int64_t* vglob, int64_t* tidx, int32_t* orient, int32_t* barrier,
                                               int64_t cap_v, int64_t cap_t, int32_t cap_m) {
    try {
        const omg::HostGeometry h = omg::load_geometry_files(geom, cond);
        const int64_t s[6] = {h.nmesh, h.nv, h.nvg, h.nt, h.N, h.nP};
        for (int i = 0; i < 6; ++i) sizes[i] = s[i];
        if (cap_v >= h.nv && cap_t >= h.nt && cap_m >= h.nmesh) {
            for (int64_t i = 0; i < 3 * h.nv; ++i) V[i] = h.V[i];
            for (int64_t i = 0; i < h.nv; ++i) vglob[i] = h.vglob[i];
            for (int64_t i = 0; i < h.nt; ++i) tidx[i] = h.tidx[i];
            for (int m = 0; m < h.nmesh; ++m) {
                orient[m] = h.orient[m];
                barrier[m] = h.barrier[m];
            }
        }
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}
