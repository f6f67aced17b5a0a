"""Seeded synthetic head models, dipoles and sensors.

Nested icosphere heads stand in for segmented MRI surfaces: each surface is an
icosahedron subdivided ``subdiv`` times and projected on a sphere, optionally
perturbed radially by a smooth real spherical-harmonic field.  Dipoles are
uniform in a ball with moments uniform on the unit sphere; EEG electrodes and
MEG point magnetometers sit on Fibonacci lattices.  Triangle orientation
defaults to inward normals, the convention of OpenMEEG's sample heads
(``data/Head3/*.tri``); the geometry layer re-orients interfaces either way
(``OpenMEEG/src/interface.cpp:55-95``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "icosphere", "sh_field", "NestedHead", "nested_head", "random_dipoles",
    "fibonacci_points", "radial_magnetometers",
]


def icosphere(subdiv: int, inward: bool = True):
    """Unit icosphere: (vertices (n,3) float64, triangles (m,3) int64).

    ``subdiv`` = 0..6; vertex count 10*4**subdiv + 2, triangles 20*4**subdiv.
    """
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
             (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    V = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in verts]
    F = faces
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = V[a] + V[b]
                V.append(m / np.linalg.norm(m))
                cache[key] = len(V) - 1
            return cache[key]

        nf = []
        for a, b, c in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = nf
    verts = np.array(V, dtype=np.float64)
    tris = np.array(F, dtype=np.int64)
    # The faces above have outward normals ((b-a)x(c-a) points away from 0).
    if inward:
        tris = tris[:, [0, 2, 1]].copy()
    return verts, tris


def _real_sh_basis(xyz: np.ndarray, lmax: int) -> np.ndarray:
    """Real spherical harmonics (unnormalised associated-Legendre form) up to lmax."""
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    r = np.linalg.norm(xyz, axis=1)
    ct = np.clip(z / r, -1.0, 1.0)
    phi = np.arctan2(y, x)
    cols = []
    for l in range(lmax + 1):
        for m in range(0, l + 1):
            # associated Legendre P_l^m(ct) by recurrence
            pmm = np.ones_like(ct)
            st = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
            for k in range(1, m + 1):
                pmm = pmm * (-(2 * k - 1)) * st
            if l == m:
                plm = pmm
            else:
                pm1 = ct * (2 * m + 1) * pmm
                if l == m + 1:
                    plm = pm1
                else:
                    a, b = pmm, pm1
                    for ll in range(m + 2, l + 1):
                        a, b = b, ((2 * ll - 1) * ct * b - (ll + m - 1) * a) / (ll - m)
                    plm = b
            norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - m) / math.factorial(l + m))
            cols.append(norm * plm * np.cos(m * phi))
            if m > 0:
                cols.append(norm * plm * np.sin(m * phi))
    return np.stack(cols, axis=1)


def sh_field(xyz: np.ndarray, seed: int, lmax: int = 4) -> np.ndarray:
    """Smooth seeded field on the sphere, degrees 1..lmax, scaled to max |f| = 1."""
    B = _real_sh_basis(xyz, lmax)[:, 1:]  # drop the constant term
    rng = np.random.default_rng(seed)
    c = rng.standard_normal(B.shape[1])
    f = B @ c
    return f / np.max(np.abs(f))


@dataclass
class NestedHead:
    """Nested closed surfaces (innermost first) with domain conductivities.

    ``domains`` follows the ``.geom`` v1.1 convention: each entry is
    ``(name, [signed 1-based interface ids], sigma)`` with ``-i`` meaning
    "inside interface i" and ``+i`` "outside interface i"
    (``OpenMEEG/include/GeometryIOs/GeomFile.h:265-300``).
    """
    vertices: list
    triangles: list
    names: list
    domains: list = field(default_factory=list)

    @property
    def n_layers(self):
        return len(self.vertices)

    def n_unknowns(self):
        # all vertices + triangles of non-barrier meshes (the outermost mesh
        # touches air and carries no triangle unknowns)
        nv = sum(v.shape[0] for v in self.vertices)
        nt = sum(t.shape[0] for t in self.triangles[:-1])
        return nv + nt


def nested_head(subdivs, radii, sigmas, perturb_seed=None, perturb_amp=0.02, lmax=4, inward=True,
                names=None) -> NestedHead:
    """Nested icosphere head.  ``sigmas`` lists the conductivity of each
    compartment from the innermost outward (len = n_layers); the region
    outside the last surface is air (sigma 0)."""
    L = len(radii)
    if isinstance(subdivs, int):
        subdivs = [subdivs] * L
    assert len(subdivs) == L and len(sigmas) == L
    assert all(radii[i] < radii[i + 1] for i in range(L - 1)), "radii must increase"
    verts, tris = [], []
    for k in range(L):
        v, t = icosphere(subdivs[k], inward=inward)
        if perturb_seed is not None:
            v = v * (1.0 + perturb_amp * sh_field(v, perturb_seed, lmax))[:, None]
        verts.append(v * radii[k])
        tris.append(t)
    if names is None:
        default = {3: ["cortex", "skull", "scalp"], 4: ["cortex", "csf", "skull", "scalp"]}
        names = default.get(L, [f"surf{k}" for k in range(L)])
    dnames = {3: ["Brain", "Skull", "Scalp"], 4: ["Brain", "CSF", "Skull", "Scalp"]}.get(
        L, [f"Dom{k}" for k in range(L)])
    domains = []
    for k in range(L):
        b = [-(k + 1)] if k == 0 else [k, -(k + 1)]
        domains.append((dnames[k], b, float(sigmas[k])))
    domains.append(("Air", [L], 0.0))
    return NestedHead(verts, tris, list(names), domains)


def random_dipoles(n: int, seed: int, rmax: float = 0.8) -> np.ndarray:
    """(n,6) dipoles: positions uniform in the ball r<rmax, unit moments uniform on S^2."""
    rng = np.random.default_rng(seed)
    u = rng.standard_normal((n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    r = rmax * rng.random(n) ** (1.0 / 3.0)
    q = rng.standard_normal((n, 3))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return np.hstack([u * r[:, None], q])


def fibonacci_points(n: int, radius: float = 1.0) -> np.ndarray:
    """(n,3) points of the Fibonacci lattice on a sphere."""
    i = np.arange(n, dtype=np.float64) + 0.5
    z = 1.0 - 2.0 * i / n
    rho = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = math.pi * (3.0 - math.sqrt(5.0)) * i
    return radius * np.stack([rho * np.cos(phi), rho * np.sin(phi), z], axis=1)


def radial_magnetometers(n: int, radius: float = 1.2) -> np.ndarray:
    """(n,6) point magnetometers: Fibonacci positions, radial unit orientations."""
    p = fibonacci_points(n, radius)
    return np.hstack([p, p / np.linalg.norm(p, axis=1, keepdims=True)])
