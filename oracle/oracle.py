"""CPU oracle for the symmetric-BEM forward path -- TEST INFRASTRUCTURE ONLY.

This module is the parity checker and the CPU baseline ("port").  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs use it; the
product (``openmeeg_gb300``) never imports it.

It restates, in Python, OpenMEEG's geometry bookkeeping for meshes given as
interfaces (``.geom`` v1.1 with one mesh per interface):

* interface orientation from the solid angle at the bounding-box centre
  (``OpenMEEG/src/interface.cpp:55-95``),
* domain/mesh orientation (``OpenMEEG/include/domain.h:43-45,95-101``),
* current barriers, outermost meshes and isolated parts
  (``OpenMEEG/src/geometry.cpp:424-536``, ``include/geometry.h:228-249``),
* unknown numbering (``OpenMEEG/src/geometry.cpp:256-295``),
* mesh pairs and S/N/D coefficients (``OpenMEEG/src/geometry.cpp:405-420``,
  ``OpenMEEG/src/assembleHeadMat.cpp:92-95``),
* dipole domain lookup (``OpenMEEG/src/geometry.cpp:146-154``,
  ``OpenMEEG/src/domain.cpp:12-17``, ``OpenMEEG/src/interface.cpp:18-35``),

and drives the C restatement of the numerical kernels in ``om_oracle.c``.
The dense solve uses LAPACK's symmetric-indefinite (Bunch-Kaufman) solver via
scipy, the same family as the reference's DSPTRF/DSPTRS
(``OpenMEEGMaths/src/symmatrix.cpp:133-152``).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libomoracle.so")
K = 1.0 / (4.0 * math.pi)


def build(force: bool = False) -> str:
    """Compile om_oracle.c (gcc, OpenMP) into oracle/_build/."""
    src = os.path.join(HERE, "om_oracle.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + f".{os.getpid()}.tmp"
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-std=c11", src, "-o", tmp,
                           "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.oo_num_threads.restype = ctypes.c_int
    return _lib


class _Geom(ctypes.Structure):
    _fields_ = [
        ("nv", ctypes.c_int64), ("V", ctypes.c_void_p), ("nt", ctypes.c_int64), ("T", ctypes.c_void_p),
        ("nmesh", ctypes.c_int), ("mesh_vbeg", ctypes.c_void_p), ("mesh_tbeg", ctypes.c_void_p),
        ("vidx", ctypes.c_void_p), ("tidx", ctypes.c_void_p), ("barrier", ctypes.c_void_p),
        ("npairs", ctypes.c_int), ("pairs", ctypes.c_void_p), ("coefs", ctypes.c_void_p),
        ("nparts", ctypes.c_int), ("part_beg", ctypes.c_void_p), ("part_meshes", ctypes.c_void_p),
        ("N", ctypes.c_int64),
    ]


class _Integ(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("levels", ctypes.c_int), ("tol", ctypes.c_double)]


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _tri_solid_angles(V, T, p):
    """Triangle::solid_angle summed over a mesh (triangle.h:123-136)."""
    r0, r1, r2 = V[T[:, 0]] - p, V[T[:, 1]] - p, V[T[:, 2]] - p
    d0, d1, d2 = (np.linalg.norm(r, axis=1) for r in (r0, r1, r2))
    nn = np.cross(V[T[:, 1]] - V[T[:, 0]], V[T[:, 2]] - V[T[:, 0]])
    nrm = np.linalg.norm(nn, axis=1)
    area = 0.5 * nrm
    n = nn / nrm[:, None]
    d = 2 * area * np.einsum("ij,ij->i", r0, n)
    den = d0 * d1 * d2 + d0 * np.einsum("ij,ij->i", r1, r2) + d1 * np.einsum("ij,ij->i", r2, r0) + \
        d2 * np.einsum("ij,ij->i", r0, r1)
    s = np.where(np.abs(d) < 1e-10, 0.0, 2 * np.arctan2(d, den))
    return float(np.sum(s))


def _almost_equal(x, y, eps=1e3):
    # om_common.h:24-26
    return abs(x - y) < np.finfo(float).eps * abs(x + y) * eps or abs(x - y) < np.finfo(float).tiny


@dataclass
class OracleGeometry:
    """Digested geometry: flat arrays plus the domain bookkeeping."""
    V: np.ndarray
    T: np.ndarray
    mesh_vbeg: np.ndarray
    mesh_tbeg: np.ndarray
    vidx: np.ndarray
    tidx: np.ndarray
    barrier: np.ndarray
    pairs: np.ndarray
    coefs: np.ndarray
    part_beg: np.ndarray
    part_meshes: np.ndarray
    N: int
    orient: np.ndarray          # per mesh (interface) orientation +-1
    domains: list               # (name, [(mesh, inside)], sigma)
    outermost: np.ndarray

    @property
    def nmesh(self):
        return len(self.mesh_tbeg) - 1

    def c_struct(self):
        g = _Geom()
        self._keep = [self.V, self.T, self.mesh_vbeg, self.mesh_tbeg, self.vidx, self.tidx, self.barrier,
                      self.pairs, self.coefs, self.part_beg, self.part_meshes]
        g.nv = self.V.shape[0]; g.V = _ptr(self.V); g.nt = self.T.shape[0]; g.T = _ptr(self.T)
        g.nmesh = self.nmesh; g.mesh_vbeg = _ptr(self.mesh_vbeg); g.mesh_tbeg = _ptr(self.mesh_tbeg)
        g.vidx = _ptr(self.vidx); g.tidx = _ptr(self.tidx); g.barrier = _ptr(self.barrier)
        g.npairs = self.pairs.shape[0]; g.pairs = _ptr(self.pairs); g.coefs = _ptr(self.coefs)
        g.nparts = len(self.part_beg) - 1; g.part_beg = _ptr(self.part_beg); g.part_meshes = _ptr(self.part_meshes)
        g.N = self.N
        return g

    # --- domain helpers -------------------------------------------------
    def mesh_orientation(self, d, m):
        for (mm, inside) in self.domains[d][1]:
            if mm == m:
                return int(self.orient[m]) if inside else -int(self.orient[m])
        return 0

    def domains_of(self, m):
        return [d for d in range(len(self.domains)) if self.mesh_orientation(d, m) != 0]

    def conductivity_jump(self, m):
        # geometry.h:188-194
        return sum(self.domains[d][2] * self.mesh_orientation(d, m) for d in self.domains_of(m))

    def interface_contains(self, m, p, sa=None):
        s = self.orient[m] * (sa if sa is not None else _tri_solid_angles(
            self.V, self.T[self.mesh_tbeg[m]:self.mesh_tbeg[m + 1]], p))
        if _almost_equal(s, -4 * math.pi):
            return True
        if _almost_equal(s, 0.0):
            return False
        if _almost_equal(s, 4 * math.pi):
            return True
        return abs(s) > 2 * math.pi

    def domain_of_point(self, p, sas=None):
        for d, (_, bounds, _) in enumerate(self.domains):
            if all(self.interface_contains(m, p, None if sas is None else sas[m]) == inside
                   for (m, inside) in bounds):
                return d
        raise ValueError("point in no domain")

    def eeg_meshes(self):
        out = []
        for (_, bounds, sigma) in self.domains:
            if sigma == 0.0:
                out += [m for (m, _) in bounds]
        return out


def digest(head) -> OracleGeometry:
    """Restate Geometry::finalize for a NestedHead-like object (vertices,
    triangles lists and .geom-style domains)."""
    nmesh = len(head.vertices)
    V = np.ascontiguousarray(np.vstack(head.vertices), dtype=np.float64)
    vbeg = np.zeros(nmesh + 1, np.int64)
    tbeg = np.zeros(nmesh + 1, np.int64)
    Ts = []
    for m in range(nmesh):
        vbeg[m + 1] = vbeg[m] + head.vertices[m].shape[0]
        tbeg[m + 1] = tbeg[m] + head.triangles[m].shape[0]
        Ts.append(np.asarray(head.triangles[m], np.int64) + vbeg[m])
    T = np.ascontiguousarray(np.vstack(Ts), dtype=np.int64)

    # interface orientation (interface.cpp:55-95): one mesh per interface
    orient = np.ones(nmesh, np.int64)
    for m in range(nmesh):
        vv = head.vertices[m]
        center = 0.5 * (vv.min(axis=0) + vv.max(axis=0))
        s = _tri_solid_angles(V, T[tbeg[m]:tbeg[m + 1]], center)
        if _almost_equal(s, 4 * math.pi):
            orient[m] = -1
            s = -s
        if not (_almost_equal(s, 0.0) or _almost_equal(s, -4 * math.pi)):
            raise ValueError(f"interface {m} is not closed (solid angle {s / math.pi} pi)")

    domains = []
    for (name, bounds, sigma) in head.domains:
        # GeomFile.h:289-291: a leading '-' means "inside"
        domains.append((name, [(abs(b) - 1, b < 0) for b in bounds], float(sigma)))
    g = OracleGeometry(V, T, vbeg, tbeg, None, None, None, None, None, None, None, 0, orient, domains, None)

    # mark_current_barriers (geometry.cpp:424-536)
    barrier = np.zeros(nmesh, np.int32)
    isolated = np.zeros(nmesh, bool)
    outermost = np.zeros(nmesh, bool)
    for (_, bounds, sigma) in domains:
        if _almost_equal(sigma, 0.0):
            for (m, _) in bounds:
                if barrier[m]:
                    isolated[m] = True
                    outermost[m] = False
                barrier[m] = 1
    for (_, bounds, sigma) in domains:
        if _almost_equal(sigma, 0.0):
            for (m, inside) in bounds:
                if not inside and barrier[m] and not isolated[m]:
                    outermost[m] = True
    # connectivity of meshes through common domains -> independent parts
    cand = list(range(nmesh))
    parts = []
    while cand:
        c = cand.pop(0)
        conn, pend = [c], [c]
        while pend:
            cur = pend.pop(0)
            keep = []
            for it in cand:
                if set(g.domains_of(cur)) & set(g.domains_of(it)):
                    conn.append(it)
                    pend.append(it)
                else:
                    keep.append(it)
            cand = keep
        if len(conn) > 1 or not isolated[conn[0]]:
            parts.append(conn)
    # outermost domain = the one with no inside boundary (geometry.cpp:23-41)
    for (_, bounds, _) in domains:
        if all(not inside for (_, inside) in bounds):
            for (m, _) in bounds:
                outermost[m] = True
            break
    if isolated.any():
        raise NotImplementedError("isolated meshes are outside this oracle's scope")

    # generate_indices (geometry.cpp:256-295)
    nv = V.shape[0]
    vidx = np.arange(nv, dtype=np.int64)
    idx = nv
    tidx = np.full(T.shape[0], -1, np.int64)
    for m in range(nmesh):
        if not barrier[m]:
            tidx[tbeg[m]:tbeg[m + 1]] = np.arange(idx, idx + tbeg[m + 1] - tbeg[m])
            idx += tbeg[m + 1] - tbeg[m]
    nbarrier_tri = 0
    for m in range(nmesh):
        if barrier[m]:
            nbarrier_tri += tbeg[m + 1] - tbeg[m]
            tidx[tbeg[m]:tbeg[m + 1]] = np.arange(idx, idx + tbeg[m + 1] - tbeg[m])
            idx += tbeg[m + 1] - tbeg[m]
    N = int(idx - nbarrier_tri)

    # make_mesh_pairs (geometry.cpp:405-420) + coefficients (assembleHeadMat.cpp:92-95)
    pairs, coefs = [], []
    for m1 in range(nmesh):
        for m2 in range(m1 + 1):
            common = sorted(set(g.domains_of(m1)) & set(g.domains_of(m2)))
            if m1 == m2:
                orientation = 1
            else:
                orientation = 0 if not common else (
                    1 if g.mesh_orientation(common[0], m1) == g.mesh_orientation(common[0], m2) else -1)
            sig = sum(domains[d][2] for d in common)
            if sig != 0.0 and orientation != 0:
                with np.errstate(divide="ignore"):
                    sinv = sum((1.0 / domains[d][2]) if domains[d][2] != 0 else np.inf for d in common)
                factor = orientation * K
                pairs.append((m1, m2))
                coefs.append((factor * sinv, factor * sig, -factor * len(common)))
    part_meshes, part_beg = [], [0]
    for part in parts:
        part_meshes += [m for m in part if outermost[m]]
        part_beg.append(len(part_meshes))

    g.vidx, g.tidx, g.barrier = vidx, tidx, barrier.astype(np.int32)
    g.pairs = np.ascontiguousarray(np.array(pairs, np.int32).reshape(-1, 2))
    g.coefs = np.ascontiguousarray(np.array(coefs, np.float64).reshape(-1, 3))
    g.part_beg = np.array(part_beg, np.int32)
    g.part_meshes = np.array(part_meshes, np.int32)
    g.N = N
    g.outermost = outermost
    return g


# ---------------------------------------------------------------------------
# Numerical entry points
# ---------------------------------------------------------------------------

def _integ(order=3, levels=0, tol=0.005):
    return _Integ(order, levels, tol)


def packed_to_dense(p: np.ndarray, n: int) -> np.ndarray:
    """Packed upper (i + j(j+1)/2) -> dense symmetric."""
    M = np.zeros((n, n))
    iu = np.triu_indices(n)
    # index of (i,j), i<=j, in packed storage
    M[iu] = p[iu[0] + iu[1] * (iu[1] + 1) // 2]
    return M + np.triu(M, 1).T


def headmat_packed(g: OracleGeometry, order=3, levels=0, tol=0.005) -> np.ndarray:
    out = np.zeros(g.N * (g.N + 1) // 2)
    gs = g.c_struct()
    it = _integ(order, levels, tol)
    lib().oo_headmat(ctypes.byref(gs), ctypes.byref(it), _ptr(out))
    return out


def headmat(g: OracleGeometry, **kw) -> np.ndarray:
    return packed_to_dense(headmat_packed(g, **kw), g.N)


def mesh_solid_angles(g: OracleGeometry, pts: np.ndarray) -> np.ndarray:
    pts = np.ascontiguousarray(pts, np.float64)
    out = np.zeros((pts.shape[0], g.nmesh))
    gs = g.c_struct()
    lib().oo_mesh_solid_angles(ctypes.byref(gs), _ptr(pts), ctypes.c_int64(pts.shape[0]), _ptr(out))
    return out


def dipole_domains(g: OracleGeometry, dipoles: np.ndarray):
    """Per dipole: the boundary meshes of its domain, their coeffD and the
    domain conductivity (assembleSourceMat.cpp:79-98)."""
    sas = mesh_solid_angles(g, dipoles[:, :3])
    n = dipoles.shape[0]
    maxb = max(len(b) for (_, b, _) in g.domains)
    nb = np.zeros(n, np.int32)
    mesh = np.zeros((n, maxb), np.int32)
    coeff = np.zeros((n, maxb))
    cond = np.zeros(n)
    for i in range(n):
        d = g.domain_of_point(dipoles[i, :3], sas[i])
        name, bounds, sigma = g.domains[d]
        cond[i] = sigma
        k = 0
        for (m, inside) in bounds:
            factorD = -K if inside else K
            mesh[i, k] = m
            coeff[i, k] = factorD * g.orient[m]
            k += 1
        nb[i] = k
    return nb, mesh, coeff, cond, maxb


def dsm(g: OracleGeometry, dipoles: np.ndarray, order=3, levels=10, tol=0.001) -> np.ndarray:
    dipoles = np.ascontiguousarray(dipoles, np.float64)
    nb, mesh, coeff, cond, maxb = dipole_domains(g, dipoles)
    n = dipoles.shape[0]
    out = np.zeros((n, g.N))  # column-major N x n
    gs = g.c_struct()
    it = _integ(order, levels, tol)
    lib().oo_dsm(ctypes.byref(gs), _ptr(dipoles), ctypes.c_int64(n), _ptr(nb), _ptr(np.ascontiguousarray(mesh)),
                 _ptr(np.ascontiguousarray(coeff)), _ptr(cond), ctypes.c_int(maxb), ctypes.byref(it), _ptr(out))
    return out.T.copy()


def _kept_points(g: OracleGeometry, points: np.ndarray):
    """Points outside zero-conductivity domains, in input order
    (assembleHeadMat.cpp:331-340, assembleSourceMat.cpp:158-170), with the
    index of the domain of each (Geometry::domain, geometry.cpp:146-154)."""
    pts = np.ascontiguousarray(points, np.float64)[:, :3]
    sas = mesh_solid_angles(g, pts)
    doms = np.array([g.domain_of_point(pts[i], sas[i]) for i in range(pts.shape[0])], np.int64)
    keep = np.array([g.domains[d][2] != 0.0 for d in doms], bool)
    return np.ascontiguousarray(pts[keep]), doms[keep]


def surf2volmat(g: OracleGeometry, points: np.ndarray) -> np.ndarray:
    """Surf2VolMat (assembleHeadMat.cpp:325-363): n_kept x N."""
    pts, _ = _kept_points(g, points)
    nb, mesh, coeffD, cond, maxb = dipole_domains(g, pts)
    n = pts.shape[0]
    out = np.zeros((g.N, n))   # column-major n x N
    gs = g.c_struct()
    # K * mesh_orientation (domain.h:43-45) is the opposite of the DipSourceMat's factorD * orientation
    lib().oo_surf2vol(ctypes.byref(gs), _ptr(pts), ctypes.c_int64(n), _ptr(nb), _ptr(np.ascontiguousarray(mesh)),
                      _ptr(np.ascontiguousarray(-coeffD)), _ptr(cond), ctypes.c_int(maxb), _ptr(out))
    return out.T.copy()


def dipsource2internalpotmat(g: OracleGeometry, dipoles: np.ndarray, points: np.ndarray,
                             domain_name: str = "") -> np.ndarray:
    """DipSource2InternalPotMat (assembleSourceMat.cpp:154-187): n_kept x n_dipoles,
    K / sigma * q.(x - r0) / |x - r0|^3 (dipole.h:29-36) where point and dipole
    share a domain."""
    pts, pdom = _kept_points(g, points)
    dip = np.asarray(dipoles, np.float64)
    if domain_name:
        ddom = np.full(dip.shape[0], [d[0] for d in g.domains].index(domain_name))
    else:
        sas = mesh_solid_angles(g, np.ascontiguousarray(dip[:, :3]))
        ddom = np.array([g.domain_of_point(dip[j, :3], sas[j]) for j in range(dip.shape[0])])
    out = np.zeros((pts.shape[0], dip.shape[0]))
    for j in range(dip.shape[0]):
        coeff = K / g.domains[ddom[j]][2]
        for i in range(pts.shape[0]):
            if pdom[i] == ddom[j]:
                x = pts[i] - dip[j, :3]
                n2 = float(x @ x)
                out[i, j] += coeff * (float(dip[j, 3:6] @ x) / (n2 * np.sqrt(n2)))
    return out


def _nearest(g: OracleGeometry, electrodes: np.ndarray):
    """Nearest triangle of the interfaces touching air (dist_point_geom,
    danielsson.cpp:107-128) and its barycentric weights, per point."""
    pos = np.ascontiguousarray(electrodes[:, :3], np.float64)
    meshes = np.array(g.eeg_meshes(), np.int32)
    ne = pos.shape[0]
    tri = np.zeros(ne, np.int64)
    w = np.zeros((ne, 3))
    gs = g.c_struct()
    lib().oo_h2em(ctypes.byref(gs), _ptr(pos), ctypes.c_int64(ne), ctypes.c_int(len(meshes)), _ptr(meshes),
                  _ptr(tri), _ptr(w))
    return tri, w


def h2em(g: OracleGeometry, electrodes: np.ndarray) -> np.ndarray:
    """Dense n_e x N Head2EEGMat (the reference stores it sparse)."""
    tri, w = _nearest(g, electrodes)
    ne = tri.shape[0]
    M = np.zeros((ne, g.N))
    for i in range(ne):
        for j in range(3):
            M[i, g.vidx[g.T[tri[i], j]]] = w[i, j]
    return M


def _tri_area(g: OracleGeometry, t) -> float:
    a, b, c = g.V[g.T[t]]
    return float(np.linalg.norm(np.cross(b - a, c - a)) / 2.0)


def injection_triangles(g: OracleGeometry, electrodes: np.ndarray):
    """Sensors::findInjectionTriangles (sensors.cpp:167-215) for electrodes
    given as n x 3 (points) or n x 4 (x, y, z, radius): per electrode the list
    of (triangle, weight) that EITSourceMat sums (assembleSourceMat.cpp:141-150).
    The walk over neighbours uses the first three entries of
    Mesh::adjacent_triangles (mesh.h:164-172), which include the triangle itself."""
    el = np.asarray(electrodes, np.float64)
    radii = el[:, 3] if el.shape[1] >= 4 else np.zeros(el.shape[0])
    nearest, _ = _nearest(g, el)
    inc = {}
    for m in range(g.nmesh):
        for t in range(g.mesh_tbeg[m], g.mesh_tbeg[m + 1]):
            for v in g.T[t]:
                inc.setdefault(int(v), []).append(t)

    def adjacent(t):
        cnt, res = {}, []
        for v in g.T[t]:
            for t2 in inc[int(v)]:
                cnt[t2] = cnt.get(t2, 0) + 1
                if cnt[t2] == 2:
                    res.append(t2)
        return res

    out = []
    for e in range(el.shape[0]):
        t0, r = int(nearest[e]), float(radii[e])
        tris = [t0]
        point = abs(r) < 2.2250738585072014e-308
        if not point and _tri_area(g, t0) < 4 * math.pi * r * r:
            seen, stack = {t0}, [t0]
            while stack:
                t = stack.pop()
                if np.linalg.norm(g.V[g.T[t]].sum(axis=0) / 3.0 - el[e, :3]) < r:
                    if t != t0:
                        tris.append(t)
                    for t2 in adjacent(t)[:3]:
                        if t2 not in seen:
                            seen.add(t2)
                            stack.append(t2)
        if point:
            out.append([(t, 1.0 / _tri_area(g, t)) for t in tris])
        else:
            w = math.pi * r * r / sum(_tri_area(g, t) for t in tris)
            out.append([(t, w) for t in tris])
    return out


def eitsourcemat(g: OracleGeometry, electrodes: np.ndarray, order=3) -> np.ndarray:
    """EITSourceMat (assembleSourceMat.cpp:109-152): N x n_electrodes."""
    inj = injection_triangles(g, electrodes)
    uniq = sorted({t for lst in inj for (t, _) in lst})
    pos = {t: k for k, t in enumerate(uniq)}
    orient = np.sign(g.coefs[:, 1])                       # the pair's relative orientation (cN = o K sigma)
    cD = np.ascontiguousarray(K * orient)
    cS = np.ascontiguousarray(-g.coefs[:, 0])             # -K o sigma_inv
    rows = np.zeros((len(uniq), g.N))
    gs = g.c_struct()
    tri = np.ascontiguousarray(np.array(uniq, np.int64))
    lib().oo_eit_rows(ctypes.byref(gs), _ptr(tri), ctypes.c_int64(len(uniq)), _ptr(cD), _ptr(cS),
                      ctypes.byref(_integ(order, 0, 0.005)), _ptr(rows))
    M = np.zeros((g.N, len(inj)))
    for e, lst in enumerate(inj):
        for (t, w) in lst:
            M[:, e] += rows[pos[t]] * w
    return M


def h2mm(g: OracleGeometry, squids: np.ndarray) -> np.ndarray:
    """n_s x N Head2MEGMat for point sensors with unit weights."""
    pos = np.ascontiguousarray(squids[:, :3], np.float64)
    ori = np.ascontiguousarray(squids[:, 3:6], np.float64)
    jump = np.array([g.conductivity_jump(m) for m in range(g.nmesh)], np.float64)
    n = pos.shape[0]
    out = np.zeros((g.N, n))
    gs = g.c_struct()
    lib().oo_h2mm(ctypes.byref(gs), _ptr(pos), _ptr(ori), ctypes.c_int64(n), _ptr(jump), _ptr(out))
    return out.T.copy()


def ds2mm(dipoles: np.ndarray, squids: np.ndarray) -> np.ndarray:
    dip = np.ascontiguousarray(dipoles, np.float64)
    pos = np.ascontiguousarray(squids[:, :3], np.float64)
    ori = np.ascontiguousarray(squids[:, 3:6], np.float64)
    out = np.zeros((dip.shape[0], pos.shape[0]))
    lib().oo_ds2mm(_ptr(dip), ctypes.c_int64(dip.shape[0]), _ptr(pos), _ptr(ori), ctypes.c_int64(pos.shape[0]),
                   _ptr(out))
    return out.T.copy()


def solve_adjoint(HM: np.ndarray, rhs_rows: np.ndarray) -> np.ndarray:
    """HM^-1 applied to the rows of `rhs_rows` (linsolve, gain.h:52-57),
    symmetric-indefinite LAPACK solve.  Returns (k x N)."""
    import scipy.linalg as sla
    return sla.solve(HM, rhs_rows.T, assume_a="sym").T


_openblas_lib = None


def _openblas():
    """scipy's bundled OpenBLAS: the BLAS/LAPACK the reference build links
    (``oracle/ref/Makefile``), with its LAPACKE entry points prefixed ``scipy_``."""
    global _openblas_lib
    if _openblas_lib is None:
        import glob

        import scipy
        d = os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs")
        cands = sorted(glob.glob(os.path.join(d, "libscipy_openblas-*.so*")))
        if not cands:
            raise RuntimeError(f"scipy's bundled OpenBLAS not found under {d}")
        lib_ = ctypes.CDLL(cands[0])
        lib_.scipy_LAPACKE_dsptrf.argtypes = [ctypes.c_int, ctypes.c_char, ctypes.c_int, ctypes.c_void_p,
                                             ctypes.c_void_p]
        lib_.scipy_LAPACKE_dsptrf.restype = ctypes.c_int
        lib_.scipy_LAPACKE_dsptrs.argtypes = [ctypes.c_int, ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        lib_.scipy_LAPACKE_dsptrs.restype = ctypes.c_int
        lib_.scipy_LAPACKE_dsptri.argtypes = [ctypes.c_int, ctypes.c_char, ctypes.c_int, ctypes.c_void_p,
                                             ctypes.c_void_p]
        lib_.scipy_LAPACKE_dsptri.restype = ctypes.c_int
        lib_.scipy_openblas_get_num_threads.restype = ctypes.c_int
        _openblas_lib = lib_
    return _openblas_lib


def openblas_threads(n: int | None = None) -> int:
    """Sets (when n is given) and returns the OpenBLAS thread count."""
    ob = _openblas()
    if n:
        ob.scipy_openblas_set_num_threads(ctypes.c_int(n))
    return int(ob.scipy_openblas_get_num_threads())


def solve_lin_packed(packed: np.ndarray, n: int, rhs: np.ndarray) -> np.ndarray:
    """SymMatrix::solveLin (OpenMEEGMaths/src/symmatrix.cpp:133-152): a copy of
    the packed-upper matrix factored by DSPTRF('U') (Bunch-Kaufman), then DSPTRS
    on the n x k right-hand sides.  Returns the n x k solution."""
    if n * (n + 1) // 2 != packed.size:
        raise ValueError("packed size does not match n")
    ob = _openblas()
    A = np.array(packed, dtype=np.float64, copy=True)
    piv = np.zeros(n, dtype=np.int32)
    info = ob.scipy_LAPACKE_dsptrf(102, b"U", n, A.ctypes.data, piv.ctypes.data)
    if info != 0:
        raise np.linalg.LinAlgError(f"DSPTRF info = {info}")
    B = np.asfortranarray(rhs, dtype=np.float64).copy(order="F")
    k = B.shape[1]
    info = ob.scipy_LAPACKE_dsptrs(102, b"U", n, k, A.ctypes.data, piv.ctypes.data, B.ctypes.data, n)
    if info != 0:
        raise np.linalg.LinAlgError(f"DSPTRS info = {info}")
    return B


def invert_packed(packed: np.ndarray, n: int) -> np.ndarray:
    """SymMatrix::invert (OpenMEEGMaths/include/symmatrix.h:280-300), what
    om_minverser runs: DSPTRF('U') then DSPTRI on packed-upper storage.
    Returns the packed-upper inverse."""
    if n * (n + 1) // 2 != packed.size:
        raise ValueError("packed size does not match n")
    ob = _openblas()
    A = np.array(packed, dtype=np.float64, copy=True)
    piv = np.zeros(n, dtype=np.int32)
    info = ob.scipy_LAPACKE_dsptrf(102, b"U", n, A.ctypes.data, piv.ctypes.data)
    if info != 0:
        raise np.linalg.LinAlgError(f"DSPTRF info = {info}")
    info = ob.scipy_LAPACKE_dsptri(102, b"U", n, A.ctypes.data, piv.ctypes.data)
    if info != 0:
        raise np.linalg.LinAlgError(f"DSPTRI info = {info}")
    return A


def gain_eeg_direct(HMinv, DSM, H2EM):
    """GainEEG (OpenMEEG/include/gain.h:69-76) as om_gain -EEG evaluates it
    (apps/gain.cpp:65-80): the sparse rows times the explicit inverse first,
    then the source matrix."""
    return (H2EM @ HMinv) @ DSM


def gain_meg_direct(HMinv, DSM, H2MM, DS2MM):
    """GainMEG (gain.h:60-67, apps/gain.cpp:105-122): DS2MM + (H2MM HMinv) DSM."""
    return DS2MM + (H2MM @ HMinv) @ DSM


def forward_pipeline(head, dipoles, electrodes=None, squids=None, clock=None):
    """The reference's time-to-gain pipeline on the CPU, stage by stage and at
    full size: ``om_assemble -HM`` (packed SymMatrix), ``-H2EM``, ``-H2MM``,
    ``-DS2MM``, then ``om_gain -EEGMEGadjoint`` (GainEEGMEGadjoint,
    OpenMEEG/include/gain.h:117-136): one DSPTRF/DSPTRS solve for the stacked
    sensor rows, the dipole sources, their contraction and DS2MM.  Returns the
    gains and the wall time of every stage."""
    import time
    clock = clock or time.perf_counter
    t = {}
    s = clock()
    g = digest(head)
    t["geometry"] = clock() - s
    s = clock()
    P = headmat_packed(g)
    t["headmat"] = clock() - s
    rows = []
    H2EM = H2MM = DS2MM = None
    if electrodes is not None:
        s = clock()
        H2EM = h2em(g, electrodes)
        t["h2em"] = clock() - s
        rows.append(H2EM)
    if squids is not None:
        s = clock()
        H2MM = h2mm(g, squids)
        t["h2mm"] = clock() - s
        s = clock()
        DS2MM = ds2mm(dipoles, squids)
        t["ds2mm"] = clock() - s
        rows.append(H2MM)
    s = clock()
    Y = solve_lin_packed(P, g.N, np.vstack(rows).T)          # N x (ne + nm)
    t["factor_solve"] = clock() - s
    del P
    s = clock()
    D = dsm(g, dipoles)
    t["dsm"] = clock() - s
    s = clock()
    G = Y.T @ D
    ne = 0 if H2EM is None else H2EM.shape[0]
    geeg = G[:ne] if H2EM is not None else None
    gmeg = G[ne:] + DS2MM if H2MM is not None else None
    t["contract"] = clock() - s
    return geeg, gmeg, t


def gain_eeg(HM, DSM, H2EM):
    """GainEEGadjoint semantics (gain.h:78-89): (HM^-1 H2EM^T)^T DSM."""
    return solve_adjoint(HM, H2EM) @ DSM


def gain_meg(HM, DSM, H2MM, DS2MM):
    return solve_adjoint(HM, H2MM) @ DSM + DS2MM


def set_threads(n: int):
    lib().oo_set_num_threads(ctypes.c_int(n))


def num_threads() -> int:
    return int(lib().oo_num_threads())


# ---------------------------------------------------------------------------
# Cortical mapping (OpenMEEG/src/assembleHeadMat.cpp:137-323)
# ---------------------------------------------------------------------------

def cortex_mesh(g: OracleGeometry, domain_name: str) -> int:
    """The single mesh of the single interface bounding `domain_name`
    (assembleHeadMat.cpp:179-183: om_error otherwise)."""
    for (name, bounds, _) in g.domains:
        if name == domain_name:
            if len(bounds) != 1:
                raise ValueError("CorticalMat: the source domain must be bounded by one interface")
            return bounds[0][0]
    raise ValueError(f"no domain {domain_name!r}")


def headmatrix_rows(g: OracleGeometry, cortex: int, order=3, extension=0):
    """HeadMatrix(geo, Cortex, integrator, extension) (assembleHeadMat.cpp:137-166):
    the head matrix with the cortex mesh's own block left out, deflated, and
    only the rows of the other meshes (their vertices, then their triangles
    unless a current barrier), in mesh order, plus `extension` zero rows."""
    keep = [p for p in range(g.pairs.shape[0]) if not (g.pairs[p, 0] == cortex and g.pairs[p, 1] == cortex)]
    saved = (g.pairs, g.coefs)
    g.pairs = np.ascontiguousarray(saved[0][keep])
    g.coefs = np.ascontiguousarray(saved[1][keep])
    try:
        HM = headmat(g, order=order)
    finally:
        g.pairs, g.coefs = saved
    rows = []
    for m in range(g.nmesh):
        if m == cortex:
            continue
        rows += [int(g.vidx[v]) for v in range(g.mesh_vbeg[m], g.mesh_vbeg[m + 1])]
        if not g.barrier[m]:
            rows += [int(g.tidx[t]) for t in range(g.mesh_tbeg[m], g.mesh_tbeg[m + 1])]
    out = np.zeros((len(rows) + extension, g.N))
    out[:len(rows)] = HM[rows]
    return out, rows


def gradient_norm2(g: OracleGeometry) -> np.ndarray:
    """Sum over the meshes of Mesh::gradient_norm2 (mesh.cpp:160-205), dense
    N x N symmetric: P1 terms on the vertices (with OpenMEEG's P1gradient,
    mesh.h:240-248, triangle edges triangle.h:86-94,154), P0 terms between
    adjacent triangles of meshes that are not outermost."""
    V, T = g.V, g.T
    A = np.zeros((g.N, g.N))

    def p1grad(p0, p1, p2):
        c = np.cross(p1, p2)
        return c / float(np.dot(p0, c))

    def area_normal(t):
        a, b, c = V[T[t]]
        nn = np.cross(b - a, c - a)
        nrm = float(np.linalg.norm(nn))
        return 0.5 * nrm, nn / nrm

    opp = ((1, 2), (2, 0), (0, 1))
    for m in range(g.nmesh):
        t0, t1 = int(g.mesh_tbeg[m]), int(g.mesh_tbeg[m + 1])
        inc = {}
        for t in range(t0, t1):
            for k in range(3):
                inc.setdefault(int(T[t, k]), []).append((t, k))
        for v in range(int(g.mesh_vbeg[m]), int(g.mesh_vbeg[m + 1])):
            i = int(g.vidx[v])
            for (t, k) in inc.get(v, []):
                a, _ = area_normal(t)
                gr = p1grad(V[v], V[T[t, opp[k][0]]], V[T[t, opp[k][1]]])
                A[i, i] += float(np.dot(gr, gr)) * a * a
        for t in range(t0, t1):
            a, _ = area_normal(t)
            for e in range(3):
                v1, v2, v3 = T[t, (e + 1) % 3], T[t, (e + 2) % 3], T[t, e]
                i1, i2 = int(g.vidx[v1]), int(g.vidx[v2])
                if i1 < i2:
                    val = float(np.dot(p1grad(V[v1], V[v2], V[v3]), p1grad(V[v2], V[v3], V[v1]))) * a * a
                    A[i1, i2] += val
                    A[i2, i1] = A[i1, i2]
        if not g.outermost[m]:
            for t in range(t0, t1):
                it = int(g.tidx[t])
                A[it, it] = 0.0
                a1, n1 = area_normal(t)
                c1 = V[T[t]].mean(axis=0)
                adj = []   # Mesh::adjacent_triangles (mesh.h:164-172): triangles sharing two vertices, t itself too
                cnt = {}
                for x in T[t]:
                    for (t2, _) in inc[int(x)]:
                        cnt[t2] = cnt.get(t2, 0) + 1
                        if cnt[t2] == 2:
                            adj.append(t2)
                for t2 in adj:
                    it2 = int(g.tidx[t2])
                    if it < it2:
                        a2, n2 = area_normal(t2)
                        c2 = V[T[t2]].sum(axis=0) / 3
                        d = c1 - c2
                        A[it, it2] += float(np.dot(n1, n2)) ** 2 / float(np.dot(d, d)) * a1 * a2
                        A[it2, it] = A[it, it2]
    return A


def _pinverse(Z: np.ndarray) -> np.ndarray:
    """Matrix::pinverse(0) (OpenMEEGMaths/src/matrix.cpp:45-80): SVD, singular
    values above max(m, n) * s_max * eps kept."""
    if Z.shape[1] > Z.shape[0]:
        return _pinverse(Z.T).T
    U, s, Vt = np.linalg.svd(Z, full_matrices=False)
    tol = max(Z.shape) * s[0] * np.finfo(float).eps
    r = int((s > tol).sum())
    if r == 0:
        return np.zeros((Z.shape[1], Z.shape[0]))
    return (Vt[:r].T / s[:r]) @ U[:, :r].T


def nullspace_projector(mat: np.ndarray) -> np.ndarray:
    """matop.h:15-32: V^T S V with S = 1 on the last Nc - Nl diagonal entries."""
    Nl = mat.shape[0]
    _, _, Vt = np.linalg.svd(mat, full_matrices=True)
    return Vt[Nl:].T @ Vt[Nl:]


def corticalmat(g: OracleGeometry, M: np.ndarray, domain_name: str, alpha=-1.0, beta=-1.0, order=3,
                projector=None):
    """CorticalMat (assembleHeadMat.cpp:168-236) for the dense Head2EEGMat M
    (n_electrodes x N): X = P pinv(P^T (M^T M + alphas RR) P) P^T M^T.
    Returns (X, P)."""
    cortex = cortex_mesh(g, domain_name)
    if projector is None:
        mat, _ = headmatrix_rows(g, cortex, order=order)
        projector = nullspace_projector(mat)
    P = projector
    RR = gradient_norm2(g)
    MM = M.T @ M
    nv = int(g.V.shape[0])
    if alpha < 0:
        alpha = np.linalg.norm(MM) / (1.0e3 * np.linalg.norm(RR[:nv, :nv]))
        beta = alpha * 50000.0
    d = np.zeros(g.N)
    d[:nv] = alpha
    for m in range(g.nmesh):
        if not g.barrier[m]:
            d[g.tidx[g.mesh_tbeg[m]:g.mesh_tbeg[m + 1]]] = beta
    Z = P.T @ (MM + d[:, None] * RR) @ P
    return P @ _pinverse(Z) @ (P.T @ M.T), P


def corticalmat2(g: OracleGeometry, M: np.ndarray, domain_name: str, gamma: float, order=3, H=None):
    """CorticalMat2 (assembleHeadMat.cpp:238-323): (G^-1 H^T (H G^-1 H^T)^-1)
    restricted to the electrode columns, H = [head-matrix rows outside the
    cortex; M], G the gradient norms with every triangle-triangle entry scaled
    by gamma once per ordered pair (gamma^2 off the diagonal, as the
    reference's loop over a symmetric matrix does).  Returns (X, H)."""
    cortex = cortex_mesh(g, domain_name)
    ne = M.shape[0]
    if H is None:
        H, _ = headmatrix_rows(g, cortex, order=order, extension=ne)
    H = H.copy()
    Nl = H.shape[0] - ne
    H[Nl:] = M
    G = gradient_norm2(g)
    for m in range(g.nmesh):
        if not g.barrier[m]:
            idx = g.tidx[g.mesh_tbeg[m]:g.mesh_tbeg[m + 1]]
            blk = np.ix_(idx, idx)
            scale = np.full((len(idx), len(idx)), gamma * gamma)
            np.fill_diagonal(scale, gamma)
            G[blk] *= scale
    Gi = np.linalg.inv(G)
    full = Gi @ H.T @ np.linalg.inv(H @ Gi @ H.T)
    return full[:, Nl:Nl + ne], H
