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
#include <cfloat>
#include <cmath>
#include <fstream>
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
        double nrm = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
        double area = 0.5 * nrm;
        double dn = (r[0][0] * nn[0] + r[0][1] * nn[1] + r[0][2] * nn[2]) / nrm;
        double dd = 2 * area * dn;
        auto dot = [&](int i, int j) { return r[i][0] * r[j][0] + r[i][1] * r[j][1] + r[i][2] * r[j][2]; };
        double den = d[0] * d[1] * d[2] + (d[0] * dot(1, 2) + d[1] * dot(2, 0) + d[2] * dot(0, 1));
        total += (std::fabs(dd) < 1e-10) ? 0.0 : 2 * std::atan2(dd, den);
    }
    return total;
}

}  // namespace

int HostGeometry::mesh_orientation(int d, int m) const {
    for (const auto& b : domains[d].bounds)
        if (b.mesh == m) return b.inside ? orient[m] : -orient[m];
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
    // Interface orientation (interface.cpp:55-95): bounding-box centre solid angle.
    orient.assign(nmesh, 1);
    for (int m = 0; m < nmesh; ++m) {
        double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
        for (int64_t v = vbeg[m]; v < vbeg[m + 1]; ++v)
            for (int k = 0; k < 3; ++k) {
                lo[k] = std::min(lo[k], V[3 * v + k]);
                hi[k] = std::max(hi[k], V[3 * v + k]);
            }
        double c[3] = {0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1]), 0.5 * (lo[2] + hi[2])};
        double s = mesh_solid_angle(*this, m, c);
        if (almost_equal(s, 4 * M_PI)) {
            orient[m] = -1;
            s = -s;
        }
        if (!(almost_equal(s, 0.0) || almost_equal(s, -4 * M_PI)))
            throw Error(OMG_ERR_INVALID, "interface " + std::to_string(m + 1) +
                                             " is not closed or its bounding-box centre lies outside it");
    }
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
        for (const auto& b : d.bounds)
            if (b.inside) ++n_in;
        if (n_in >= 2) nested = false;
    }
    // numbering (geometry.cpp:256-295)
    tidx.assign(nt, -1);
    int64_t idx = nv;
    for (int m = 0; m < nmesh; ++m)
        if (!barrier[m])
            for (int64_t t = tbeg[m]; t < tbeg[m + 1]; ++t) tidx[t] = idx++;
    nP = idx - nv;
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
    eeg_meshes.clear();
    for (const auto& d : domains)
        if (d.sigma == 0.0)
            for (const auto& b : d.bounds) eeg_meshes.push_back(b.mesh);
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

HostGeometry build_geometry(int nmesh, const int64_t* nverts, const double* verts, const int64_t* ntris,
                            const int64_t* tris, int ndom, const int32_t* nb, const int32_t* bounds,
                            const double* sigma, const std::vector<std::string>& dom_names) {
    OMG_REQUIRE(nmesh > 0 && ndom > 0, "geometry needs at least one mesh and one domain");
    HostGeometry g;
    g.nmesh = nmesh;
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
            OMG_REQUIRE(b != 0 && std::abs(b) <= nmesh, "domain boundary refers to an unknown interface");
            dom.bounds.push_back({std::abs(b) - 1, b < 0});   // GeomFile.h:289-291
        }
        g.domains.push_back(dom);
    }
    g.finalize();
    return g;
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
    std::vector<std::string> meshes;
    std::vector<std::string> dnames;
    std::vector<int32_t> nb, bounds;
    for (size_t i = 0; i < lines.size(); ++i) {
        std::istringstream is(lines[i]);
        std::string key;
        is >> key;
        if (key == "Interfaces") {
            int n;
            is >> n;
            for (int k = 0; k < n; ++k) {
                const std::string& e = lines[++i];
                std::string fn;
                auto q1 = e.find('"');
                if (q1 != std::string::npos)
                    fn = e.substr(q1 + 1, e.find('"', q1 + 1) - q1 - 1);
                else {
                    std::istringstream es(e);
                    std::string tok;
                    while (es >> tok) fn = tok;
                }
                meshes.push_back(fn.size() && fn[0] == '/' ? fn : dir + fn);
            }
        } else if (key == "Domains") {
            int n;
            is >> n;
            for (int k = 0; k < n; ++k) {
                std::string e = lines[++i];
                e = e.substr(e.find("Domain") + 6);
                std::string name, rest;
                auto c = e.find(':');
                if (c != std::string::npos) {
                    name = e.substr(0, c);
                    rest = e.substr(c + 1);
                } else {
                    std::istringstream es(e);
                    es >> name;
                    std::getline(es, rest);
                }
                name.erase(0, name.find_first_not_of(" \t"));
                name.erase(name.find_last_not_of(" \t") + 1);
                std::istringstream rs(rest);
                std::string tok;
                int cnt = 0;
                while (rs >> tok) {
                    if (tok == "shared") break;
                    bounds.push_back(std::stoi(tok));
                    ++cnt;
                }
                dnames.push_back(name);
                nb.push_back(cnt);
            }
        }
    }
    if (meshes.empty() || dnames.empty()) throw Error(OMG_ERR_IO, "no interfaces or domains in " + geom);
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
    for (const auto& m : meshes) {
        std::vector<double> v;
        std::vector<int64_t> t;
        read_tri(m, v, t);
        V.insert(V.end(), v.begin(), v.end());
        T.insert(T.end(), t.begin(), t.end());
        nv.push_back((int64_t)v.size() / 3);
        nt.push_back((int64_t)t.size() / 3);
    }
    return build_geometry((int)meshes.size(), nv.data(), V.data(), nt.data(), T.data(), (int)dnames.size(), nb.data(),
                          bounds.data(), sigma.data(), dnames);
}

}  // namespace omg
