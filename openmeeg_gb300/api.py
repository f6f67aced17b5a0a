"""Python mirror of OpenMEEG's forward-path API on the GB300 library.

Names and argument meanings follow the reference's Python module
(``wrapping/python/openmeeg/__init__.py:15-39``, SWIG over
``OpenMEEG/include/assemble.h``, ``assembleSourceMat.h``, ``gain.h``):
``Geometry``, ``Integrator``, ``HeadMat``, ``DipSourceMat``, ``Head2EEGMat``,
``Head2MEGMat``, ``DipSource2MEGMat``, ``GainEEG``, ``GainMEG``,
``GainEEGadjoint``, ``GainMEGadjoint``, ``GainEEGMEGadjoint``.  Matrices are
returned as float64 torch tensors on the CUDA device (``.cpu().numpy()`` gives
the reference's numpy view); inputs may be numpy arrays or tensors.  Errors
raise ``OMGError`` carrying the C status, where the reference raises its
``OpenMEEG::Exception`` hierarchy.
"""
from __future__ import annotations

import ctypes
import math
import sys
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib
from ._lib import GainStats, GeometryInfo, Integrator, OMGError, check

__all__ = ["Context", "Geometry", "Integrator", "HeadMat", "HeadMatPacked", "DipSourceMat", "Head2EEGMat",
           "Head2MEGMat", "DipSource2MEGMat", "Solver", "GainEEG", "GainMEG", "GainEEGadjoint", "GainMEGadjoint",
           "GainEEGMEGadjoint", "forward_gain", "BatchForward", "SurfSourceMat", "SurfSource2MEGMat", "Surf2VolMat",
           "DipSource2InternalPotMat", "EITSourceMat", "OMGError",
           "kernel_launches"]

FP64 = "fp64"
MIXED = "mixed"


def _prec(p) -> int:
    if p in (FP64, _lib.PREC_FP64, None):
        return _lib.PREC_FP64
    if p in (MIXED, _lib.PREC_MIXED):
        return _lib.PREC_MIXED
    raise ValueError(f"unknown precision {p!r}")


class Context:
    """A CUDA device + stream for the library (one per device and thread)."""

    _default = {}

    def __init__(self, device: int = 0):
        self.device = device
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        check(self.lib.omg_context_create(device, ctypes.byref(h)))
        self.handle = h

    @classmethod
    def default(cls, device: Optional[int] = None) -> "Context":
        if device is None:
            device = torch.cuda.current_device() if torch.cuda.is_available() else 0
        if device not in cls._default:
            cls._default[device] = cls(device)
        return cls._default[device]

    def bind_current_stream(self):
        """Queue library work on torch's current stream of this device."""
        s = torch.cuda.current_stream(self.device)
        check(self.lib.omg_context_set_stream(self.handle, ctypes.c_void_p(s.cuda_stream)))

    def synchronize(self):
        check(self.lib.omg_context_synchronize(self.handle))

    def launches(self) -> int:
        return int(self.lib.omg_context_kernel_launches(self.handle))

    def __del__(self):
        # At interpreter shutdown the process is going away; leave the
        # handles to the OS rather than racing the CUDA runtime's teardown.
        if sys.is_finalizing():
            return
        try:
            if getattr(self, "handle", None):
                self.lib.omg_context_destroy(self.handle)
        except Exception:
            pass


def kernel_launches(ctx: Optional[Context] = None) -> int:
    return (ctx or Context.default()).launches()


def _dev(ctx: Context):
    return torch.device("cuda", ctx.device)


def _as_dev(x, ctx: Context, cols: Optional[int] = None) -> torch.Tensor:
    t = torch.as_tensor(np.asarray(x) if not isinstance(x, torch.Tensor) else x, dtype=torch.float64)
    t = t.to(_dev(ctx)).contiguous()
    if cols is not None:
        if t.ndim != 2 or t.shape[1] < cols:
            raise ValueError(f"expected an (n, {cols}) array")
        if t.shape[1] != cols:
            t = t[:, :cols].contiguous()
    return t


def _ptr(t: Optional[torch.Tensor]):
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else ctypes.c_void_p(0)


class Geometry:
    """Geometry(geom_file, cond_file) or Geometry.from_meshes(...)
    (OpenMEEG/include/geometry.h:67).  Meshes are interfaces of a
    ``.geom`` v1.1 description; domains carry conductivities."""

    def __init__(self, geom_file: Optional[str] = None, cond_file: Optional[str] = None, ctx: Optional[Context] = None,
                 _handle=None):
        self.ctx = ctx or Context.default()
        self.lib = self.ctx.lib
        if _handle is not None:
            self.handle = _handle
        else:
            if geom_file is None or cond_file is None:
                raise ValueError("Geometry needs a .geom and a .cond file (or use Geometry.from_meshes)")
            h = ctypes.c_void_p()
            check(self.lib.omg_geometry_load(self.ctx.handle, geom_file.encode(), cond_file.encode(), ctypes.byref(h)))
            self.handle = h
        self.domain_names = None
        if _handle is None:   # the domains in the .geom file's order, as the library numbers them
            from . import io
            self.domain_names = [d[0] for d in io.read_geom_full(geom_file)[2]]

    @classmethod
    def from_meshes(cls, vertices: Sequence[np.ndarray], triangles: Sequence[np.ndarray], domains,
                    ctx: Optional[Context] = None) -> "Geometry":
        """domains: list of (name, [signed 1-based interface ids], sigma)."""
        ctx = ctx or Context.default()
        nv = np.array([np.asarray(v).shape[0] for v in vertices], np.int64)
        nt = np.array([np.asarray(t).shape[0] for t in triangles], np.int64)
        V = np.ascontiguousarray(np.vstack([np.asarray(v, np.float64) for v in vertices]))
        T = np.ascontiguousarray(np.vstack([np.asarray(t, np.int64) for t in triangles]))
        nb = np.array([len(d[1]) for d in domains], np.int32)
        bounds = np.array([b for d in domains for b in d[1]], np.int32)
        sig = np.array([float(d[2]) for d in domains], np.float64)
        h = ctypes.c_void_p()
        P = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))
        check(ctx.lib.omg_geometry_create(ctx.handle, len(vertices), P(nv, ctypes.c_int64), P(V, ctypes.c_double),
                                          P(nt, ctypes.c_int64), P(T, ctypes.c_int64), len(domains),
                                          P(nb, ctypes.c_int32), P(bounds, ctypes.c_int32), P(sig, ctypes.c_double),
                                          ctypes.byref(h)))
        g = cls(ctx=ctx, _handle=h)
        g.domain_names = [d[0] for d in domains]
        g._sigmas = sig
        return g

    @classmethod
    def from_head(cls, head, ctx: Optional[Context] = None) -> "Geometry":
        return cls.from_meshes(head.vertices, head.triangles, head.domains, ctx)

    def info(self) -> GeometryInfo:
        i = GeometryInfo()
        check(self.lib.omg_geometry_get_info(self.handle, ctypes.byref(i)))
        return i

    def nb_parameters(self) -> int:
        return int(self.info().n_unknowns)

    @property
    def size(self) -> int:
        return self.nb_parameters()

    def set_conductivities(self, sigmas):
        s = np.ascontiguousarray(np.asarray(sigmas, np.float64))
        check(self.lib.omg_geometry_set_conductivities(self.handle, s.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        self._sigmas = s

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            if getattr(self, "handle", None):
                self.lib.omg_geometry_destroy(self.handle)
        except Exception:
            pass


def _default(integ, order, levels, tol):
    return integ if integ is not None else Integrator(order, levels, tol)


def HeadMat(geom: Geometry, integrator: Optional[Integrator] = None, precision=FP64) -> torch.Tensor:
    """HeadMat(geo, Integrator(3,0,0.005)) (assembleHeadMat.cpp:133-135): dense N x N (both halves)."""
    ctx = geom.ctx
    N = geom.size
    out = torch.empty((N, N), dtype=torch.float64, device=_dev(ctx))
    it = _default(integrator, 3, 0, 0.005)
    check(ctx.lib.omg_headmat_dev(ctx.handle, geom.handle, ctypes.byref(it), _prec(precision), _ptr(out), N))
    return out   # symmetric: column-major == row-major


def HeadMatPacked(geom: Geometry, integrator: Optional[Integrator] = None) -> torch.Tensor:
    """HeadMat in SymMatrix packed-upper storage (what a .bin SymMatrix holds)."""
    ctx = geom.ctx
    N = geom.size
    out = torch.empty(N * (N + 1) // 2, dtype=torch.float64, device=_dev(ctx))
    it = _default(integrator, 3, 0, 0.005)
    check(ctx.lib.omg_headmat_packed_dev(ctx.handle, geom.handle, ctypes.byref(it), _ptr(out)))
    return out


def _domain_index(geom: Geometry, domain_name: str) -> int:
    """-1 for "" (each source's own domain), else the index of the named domain."""
    if not domain_name:
        return -1
    if geom.domain_names is None or domain_name not in geom.domain_names:
        raise OMGError(-1, f"unknown domain {domain_name!r}")
    return geom.domain_names.index(domain_name)


def DipSourceMat(geom: Geometry, dipoles, integrator: Optional[Integrator] = None, domain_name: str = "",
                 adaptive: bool = True) -> torch.Tensor:
    """SourceMatrix<Dipole>(geo, dipoles, Integrator(3,10,0.001), domain) (assembleSourceMat.cpp:66-104).
    Returns N x n_dipoles.  ``adaptive=False`` is om_assemble's -DSMNA (levels 0)."""
    ctx = geom.ctx
    d = _as_dev(dipoles, ctx, 6)
    n = d.shape[0]
    N = geom.size
    out = torch.empty((n, N), dtype=torch.float64, device=_dev(ctx))   # column-major N x n
    it = _default(integrator, 3, 10 if adaptive else 0, 0.001)
    dom = _domain_index(geom, domain_name)
    check(ctx.lib.omg_dipsourcemat_dev(ctx.handle, geom.handle, _ptr(d), n, ctypes.byref(it), dom, _ptr(out)))
    return out.T


def Head2EEGMat(geom: Geometry, electrodes, sparse: bool = False):
    """Head2EEGMat (assembleSensors.cpp:25-39): n_e x N (3 nonzeros per row).
    With sparse=True also returns (columns (n_e x 3), values (n_e x 3))."""
    ctx = geom.ctx
    e = _as_dev(electrodes, ctx, 3)
    n = e.shape[0]
    N = geom.size
    out = torch.empty((N, n), dtype=torch.float64, device=_dev(ctx))   # column-major n x N
    cols = torch.empty((n, 3), dtype=torch.int64, device=_dev(ctx))
    vals = torch.empty((n, 3), dtype=torch.float64, device=_dev(ctx))
    check(ctx.lib.omg_head2eegmat_dev(ctx.handle, geom.handle, _ptr(e), n, _ptr(out), _ptr(cols), _ptr(vals)))
    return (out.T, cols, vals) if sparse else out.T


def Head2MEGMat(geom: Geometry, squids) -> torch.Tensor:
    """Head2MEGMat (assembleSensors.cpp:69-96) for point sensors (n x 6: position, orientation)."""
    ctx = geom.ctx
    s = _as_dev(squids, ctx, 6)
    n = s.shape[0]
    N = geom.size
    out = torch.empty((N, n), dtype=torch.float64, device=_dev(ctx))
    check(ctx.lib.omg_head2megmat_dev(ctx.handle, geom.handle, _ptr(s), n, _ptr(out)))
    return out.T


def DipSource2MEGMat(dipoles, squids, ctx: Optional[Context] = None) -> torch.Tensor:
    """DipSource2MEGMat (assembleSensors.cpp:133-159): n_squids x n_dipoles."""
    ctx = ctx or Context.default()
    d = _as_dev(dipoles, ctx, 6)
    s = _as_dev(squids, ctx, 6)
    out = torch.empty((d.shape[0], s.shape[0]), dtype=torch.float64, device=_dev(ctx))
    check(ctx.lib.omg_dipsource2megmat_dev(ctx.handle, _ptr(d), d.shape[0], _ptr(s), s.shape[0], _ptr(out)))
    return out.T


def _mesh_arrays(vertices, triangles):
    V = np.ascontiguousarray(np.asarray(vertices, np.float64)[:, :3])
    T = np.ascontiguousarray(np.asarray(triangles, np.int64)[:, :3])
    return V, T


def SurfSourceMat(geom: Geometry, vertices, triangles, integrator: Optional[Integrator] = None) -> torch.Tensor:
    """SurfSourceMat(geo, source_mesh, integrator) (assembleSourceMat.cpp:22-64): N x n_vertices for a
    triangulated source surface inside one conducting domain."""
    V, T = _mesh_arrays(vertices, triangles)
    it = _default(integrator, 3, 0, 0.005)
    out = torch.empty((V.shape[0], geom.size), dtype=torch.float64, device=_dev(geom.ctx))   # column-major
    P = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))
    check(geom.lib.omg_surfsourcemat_dev(geom.ctx.handle, geom.handle, P(V, ctypes.c_double), V.shape[0],
                                         P(T, ctypes.c_int64), T.shape[0], ctypes.byref(it), _ptr(out)))
    return out.T


def SurfSource2MEGMat(vertices, triangles, squids, ctx: Optional[Context] = None) -> torch.Tensor:
    """SurfSource2MEGMat(source_mesh, sensors) (assembleSensors.cpp:102-125): n_squids x n_vertices."""
    ctx = ctx or Context.default()
    V, T = _mesh_arrays(vertices, triangles)
    sq = _as_dev(squids, ctx, 6)
    out = torch.empty((V.shape[0], sq.shape[0]), dtype=torch.float64, device=_dev(ctx))
    P = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))
    check(ctx.lib.omg_surfsource2megmat_dev(ctx.handle, P(V, ctypes.c_double), V.shape[0], P(T, ctypes.c_int64),
                                            T.shape[0], _ptr(sq), sq.shape[0], _ptr(out)))
    return out.T


def _kept_rows(buf: torch.Tensor, n_kept: int, cols: int) -> torch.Tensor:
    """The n_kept x cols column-major matrix at the start of ``buf``."""
    return buf[:n_kept * cols].view(cols, n_kept).T


def Surf2VolMat(geom: Geometry, points) -> torch.Tensor:
    """Surf2VolMat(geo, points) (assembleHeadMat.cpp:325-363): n_kept x N, the
    potential at points inside the head from the surface unknowns.  Points in a
    zero-conductivity domain are dropped (rows keep the input order)."""
    ctx = geom.ctx
    p = _as_dev(points, ctx, 3)
    N = geom.size
    buf = torch.empty(max(p.shape[0] * N, 1), dtype=torch.float64, device=_dev(ctx))
    kept = ctypes.c_int64()
    check(ctx.lib.omg_surf2volmat_dev(ctx.handle, geom.handle, _ptr(p), p.shape[0], _ptr(buf), ctypes.byref(kept)))
    return _kept_rows(buf, kept.value, N)


def DipSource2InternalPotMat(geom: Geometry, dipoles, points, domain_name: str = "") -> torch.Tensor:
    """DipSource2InternalPotMat(geo, dipoles, points, domain_name) (assembleSourceMat.cpp:154-187):
    n_kept x n_dipoles, the infinite-medium potential of each dipole at the
    kept points of its domain."""
    ctx = geom.ctx
    d = _as_dev(dipoles, ctx, 6)
    p = _as_dev(points, ctx, 3)
    dom = _domain_index(geom, domain_name)
    buf = torch.empty(max(p.shape[0] * d.shape[0], 1), dtype=torch.float64, device=_dev(ctx))
    kept = ctypes.c_int64()
    check(ctx.lib.omg_dipsource2internalpotmat_dev(ctx.handle, geom.handle, _ptr(d), d.shape[0], _ptr(p), p.shape[0],
                                                   dom, _ptr(buf), ctypes.byref(kept)))
    return _kept_rows(buf, kept.value, d.shape[0])


def EITSourceMat(geom: Geometry, electrodes, integrator: Optional[Integrator] = None) -> torch.Tensor:
    """EITSourceMat(geo, electrodes, integrator) (assembleSourceMat.cpp:109-152): N x n_electrodes.
    ``electrodes`` is n x 3 (point electrodes) or n x 4 (x, y, z, radius), as
    the columns of an EIT sensors file (sensors.cpp:99-108)."""
    ctx = geom.ctx
    e = _as_dev(electrodes, ctx)
    if e.ndim != 2 or e.shape[1] not in (3, 4):
        raise OMGError(-1, "electrodes must be n x 3 or n x 4 (x, y, z, radius)")
    pos = e[:, :3].contiguous()
    rad = e[:, 3].contiguous() if e.shape[1] == 4 else None
    it = _default(integrator, 3, 0, 0.005)
    out = torch.empty((e.shape[0], geom.size), dtype=torch.float64, device=_dev(ctx))   # column-major
    check(ctx.lib.omg_eitsourcemat_dev(ctx.handle, geom.handle, _ptr(pos), _ptr(rad), e.shape[0], ctypes.byref(it),
                                       _ptr(out)))
    return out.T


class Solver:
    """Factorization of the HeadMat (replaces SymMatrix::solveLin / linsolve,
    symmatrix.cpp:133-152, gain.h:52-57)."""

    def __init__(self, geom: Geometry, precision=FP64, integrator: Optional[Integrator] = None, hm=None):
        self.geom = geom
        self.ctx = geom.ctx
        h = ctypes.c_void_p()
        if hm is None:
            it = _default(integrator, 3, 0, 0.005)
            check(self.ctx.lib.omg_solver_create(self.ctx.handle, geom.handle, ctypes.byref(it), _prec(precision),
                                                 ctypes.byref(h)))
        else:
            A = _as_dev(hm, self.ctx)
            check(self.ctx.lib.omg_solver_from_headmat_dev(self.ctx.handle, geom.handle, _ptr(A), A.shape[0],
                                                           _prec(precision), ctypes.byref(h)))
        self.handle = h

    def set_refinement(self, tol: float = 1e-6, max_steps: int = 10) -> None:
        """Mixed precision: stop refining when the predicted relative error is
        below tol, after at most max_steps residual steps; a refinement that
        stalls above tol falls back to an FP64 solve of the rebuilt head matrix."""
        check(self.ctx.lib.omg_solver_set_refinement(self.handle, float(tol), int(max_steps)))

    def solve(self, B) -> torch.Tensor:
        """HM^-1 B for B of shape (N,) or (N, k)."""
        b = _as_dev(B, self.ctx)
        vec = b.ndim == 1
        if vec:
            b = b[:, None]
        X = b.T.contiguous()   # column-major N x k
        check(self.ctx.lib.omg_solver_solve_dev(self.handle, _ptr(X), b.shape[0], b.shape[1]))
        X = X.T
        return X[:, 0] if vec else X

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            if getattr(self, "handle", None):
                self.ctx.lib.omg_solver_destroy(self.handle)
        except Exception:
            pass


def forward_gain(geom: Geometry, dipoles, electrodes=None, squids=None, precision=FP64,
                 hm_integrator: Optional[Integrator] = None, dsm_integrator: Optional[Integrator] = None,
                 host: bool = False, out=None):
    """Adjoint gain pipeline (gain.h:78-136) in one call.  Returns
    (G_eeg or None, G_meg or None, stats dict).  host=True goes through the
    host-buffer entry point (copies included); there `out` may give the two
    C-contiguous float64 host arrays (n_dipoles x n_electrodes,
    n_dipoles x n_squids) the gains are written to -- pinned memory makes the
    device-to-host copies direct."""
    ctx = geom.ctx
    dip = np.ascontiguousarray(np.asarray(dipoles, np.float64)[:, :6]) if host else _as_dev(dipoles, ctx, 6)
    nd = dip.shape[0]
    ne = 0 if electrodes is None else len(electrodes)
    nm = 0 if squids is None else len(squids)
    st = GainStats()
    hi = _default(hm_integrator, 3, 0, 0.005)
    di = _default(dsm_integrator, 3, 10, 0.001)
    if host:
        el = np.ascontiguousarray(np.asarray(electrodes, np.float64)[:, :3]) if ne else np.zeros((0, 3))
        sq = np.ascontiguousarray(np.asarray(squids, np.float64)[:, :6]) if nm else np.zeros((0, 6))
        if out is not None:
            ge, gm = out
            for a, c in ((ge, ne), (gm, nm)):
                if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.shape == (nd, c)
                        and a.flags.c_contiguous):
                    raise ValueError("out: C-contiguous float64 arrays of shape (n_dipoles, n_sensors)")
        else:
            ge = np.empty((nd, ne))   # column-major ne x nd, every entry written by the library
            gm = np.empty((nd, nm))
        P = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        check(ctx.lib.omg_gain_host(ctx.handle, geom.handle, _prec(precision), ctypes.byref(hi), ctypes.byref(di),
                                    P(dip), nd, P(el), ne, P(sq), nm, P(ge), P(gm), ctypes.byref(st)))
        return (ge.T if ne else None), (gm.T if nm else None), st.as_dict()
    el = _as_dev(electrodes, ctx, 3) if ne else None
    sq = _as_dev(squids, ctx, 6) if nm else None
    ge = torch.empty((nd, ne), dtype=torch.float64, device=_dev(ctx)) if ne else None
    gm = torch.empty((nd, nm), dtype=torch.float64, device=_dev(ctx)) if nm else None
    check(ctx.lib.omg_gain_dev(ctx.handle, geom.handle, _prec(precision), ctypes.byref(hi), ctypes.byref(di),
                               _ptr(dip), nd, _ptr(el), ne, _ptr(sq), nm, _ptr(ge), _ptr(gm), ctypes.byref(st)))
    return (ge.T if ne else None), (gm.T if nm else None), st.as_dict()


class _DevView:
    """__cuda_array_interface__ over library-owned device memory (read-only use)."""

    def __init__(self, ptr: int, shape):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f8", "data": (int(ptr), False),
                                         "version": 3, "strides": None}


class BatchForward:
    """Forward gains of many head models as one captured CUDA graph (no
    reference counterpart).  Each model's gains are those of forward_gain
    (the adjoint form of gain.h:78-136) in the same precision; the models run
    as parallel branches of the graph, the branch count timed and chosen at
    construction when n_branches = 0.

    models: sequence of (Geometry, dipoles (n x 6), electrodes (n x 3) or None,
    squids (n x 6) or None), all on this context's device."""

    def __init__(self, models, precision=MIXED, n_branches: int = 0, ctx: Optional[Context] = None):
        self.ctx = ctx or models[0][0].ctx
        self.lib = self.ctx.lib
        self._keep = []
        arr = (_lib.BatchModel * len(models))()
        self.shapes = []
        for i, (geo, dip, el, sq) in enumerate(models):
            d = np.ascontiguousarray(np.asarray(dip, np.float64)[:, :6])
            e = np.ascontiguousarray(np.asarray(el, np.float64)[:, :3]) if el is not None and len(el) else None
            q = np.ascontiguousarray(np.asarray(sq, np.float64)[:, :6]) if sq is not None and len(sq) else None
            self._keep += [geo, d, e, q]
            P = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None
            arr[i] = _lib.BatchModel(geo.handle, P(d), d.shape[0], P(e), 0 if e is None else e.shape[0], P(q),
                                     0 if q is None else q.shape[0])
            self.shapes.append((d.shape[0], 0 if e is None else e.shape[0], 0 if q is None else q.shape[0]))
        h = ctypes.c_void_p()
        check(self.lib.omg_batch_create(self.ctx.handle, len(models), arr, _prec(precision), int(n_branches),
                                        ctypes.byref(h)))
        self.handle = h

    def __len__(self):
        return len(self.shapes)

    def run(self):
        """Replay the graph: every model's gains are recomputed from its inputs."""
        check(self.lib.omg_batch_run(self.handle))

    def gains(self, i: int):
        """(EEG gain n_electrodes x n_dipoles or None, MEG gain or None), copies."""
        nd, ne, nm = self.shapes[i]
        pe, pm = ctypes.c_void_p(), ctypes.c_void_p()
        check(self.lib.omg_batch_gain_dev(self.handle, i, ctypes.byref(pe), ctypes.byref(pm)))
        dev = _dev(self.ctx)
        ge = torch.as_tensor(_DevView(pe.value, (nd, ne)), device=dev).T.clone() if ne and nd else None
        gm = torch.as_tensor(_DevView(pm.value, (nd, nm)), device=dev).T.clone() if nm and nd else None
        return ge, gm

    def set_dipoles(self, i: int, dipoles):
        d = np.ascontiguousarray(np.asarray(dipoles, np.float64)[:, :6])
        if d.shape[0] != self.shapes[i][0]:
            raise ValueError("a model's dipole count is fixed at construction")
        check(self.lib.omg_batch_set_dipoles(self.handle, i, d.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))

    def info(self) -> dict:
        inf = _lib.BatchInfo()
        check(self.lib.omg_batch_get_info(self.handle, ctypes.byref(inf)))
        return inf.as_dict()

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            if getattr(self, "handle", None):
                self.lib.omg_batch_destroy(self.handle)
        except Exception:
            pass


# ---- reference class names (gain.h:60-136) --------------------------------

def _inverse_operand(HMinv, ctx: Context):
    """(device tensor, N, ld, packed): a dense N x N inverse in column-major
    order, or a 1-D SymMatrix packed-upper array of N(N+1)/2 entries."""
    t = HMinv if isinstance(HMinv, torch.Tensor) else torch.as_tensor(np.asarray(HMinv))
    t = t.to(_dev(ctx), torch.float64)
    if t.ndim == 1:
        n = int((math.isqrt(8 * t.numel() + 1) - 1) // 2)
        if n * (n + 1) // 2 != t.numel():
            raise ValueError("packed inverse: length is not N(N+1)/2")
        return t.contiguous(), n, n, 1
    if t.ndim != 2 or t.shape[0] != t.shape[1]:
        raise ValueError("inverse head matrix must be N x N or packed")
    return t.T.contiguous(), t.shape[0], t.shape[0], 0     # row-major storage of t^T = column-major t


def _cols_dev(M, ctx: Context, rows: int) -> torch.Tensor:
    """An (rows x n) matrix as a column-major device buffer (n x rows contiguous)."""
    t = M if isinstance(M, torch.Tensor) else torch.as_tensor(np.asarray(M))
    t = t.to(_dev(ctx), torch.float64)
    if t.ndim != 2 or t.shape[0] != rows:
        raise ValueError(f"expected a matrix with {rows} rows")
    return t.T.contiguous()


def _sparse_rows(H2EM, ctx: Context, N: int):
    """(n_rows, rows, cols, vals) device triplets of a sparse sensor matrix given
    dense (n x N), as a torch sparse tensor, or as the (dense, columns, values)
    triple Head2EEGMat(sparse=True) returns."""
    dev = _dev(ctx)
    if isinstance(H2EM, tuple):
        cols, vals = H2EM[1], H2EM[2]
        cols = torch.as_tensor(cols).to(dev, torch.int64)
        vals = torch.as_tensor(vals).to(dev, torch.float64)
        n = cols.shape[0]
        rows = torch.arange(n, device=dev, dtype=torch.int64)[:, None].expand_as(cols)
        return n, rows.reshape(-1).contiguous(), cols.reshape(-1).contiguous(), vals.reshape(-1).contiguous()
    t = H2EM if isinstance(H2EM, torch.Tensor) else torch.as_tensor(np.asarray(H2EM))
    if t.is_sparse:
        t = t.coalesce()
        idx = t.indices().to(dev, torch.int64)
        return t.shape[0], idx[0].contiguous(), idx[1].contiguous(), t.values().to(dev, torch.float64).contiguous()
    t = t.to(dev, torch.float64)
    if t.ndim != 2 or t.shape[1] != N:
        raise ValueError(f"sensor matrix must have {N} columns")
    nz = torch.nonzero(t, as_tuple=True)
    return t.shape[0], nz[0].contiguous(), nz[1].contiguous(), t[nz].contiguous()


def GainEEG(HMinv, DSM, H2EM, precision=FP64, ctx: Optional[Context] = None) -> torch.Tensor:
    """GainEEG(HeadMatInv, SourceMat, Head2EEGMat) = (H2EM HMinv) DSM
    (gain.h:69-76, om_gain -EEG) on the library's kernels.  HMinv: N x N or
    SymMatrix packed upper; H2EM: dense, torch sparse, or Head2EEGMat(...,
    sparse=True)'s triple.  Returns n_electrodes x n_dipoles."""
    ctx = ctx or Context.default()
    H, N, ld, packed = _inverse_operand(HMinv, ctx)
    D = _cols_dev(DSM, ctx, N)
    ne, r, c, v = _sparse_rows(H2EM, ctx, N)
    nd = D.shape[0]
    out = torch.empty((nd, ne), dtype=torch.float64, device=_dev(ctx))   # column-major ne x nd
    check(ctx.lib.omg_gain_eeg_dev(ctx.handle, N, _ptr(H), ld, packed, _ptr(D), nd, ne, r.numel(), _ptr(r), _ptr(c),
                                   _ptr(v), _prec(precision), _ptr(out)))
    return out.T


def GainMEG(HMinv, DSM, H2MM, DS2MM, precision=FP64, ctx: Optional[Context] = None) -> torch.Tensor:
    """GainMEG(HeadMatInv, SourceMat, Head2MEGMat, Source2MEGMat) =
    DS2MM + (H2MM HMinv) DSM (gain.h:60-67, om_gain -MEG) on the library's
    kernels.  Returns n_squids x n_dipoles."""
    ctx = ctx or Context.default()
    H, N, ld, packed = _inverse_operand(HMinv, ctx)
    D = _cols_dev(DSM, ctx, N)
    nd = D.shape[0]
    V = torch.as_tensor(H2MM if isinstance(H2MM, torch.Tensor) else np.asarray(H2MM)).to(_dev(ctx), torch.float64)
    nm = V.shape[0]
    if V.ndim != 2 or V.shape[1] != N:
        raise ValueError(f"Head2MEGMat must have {N} columns")
    Vc = V.T.contiguous()                                  # column-major nm x N
    S = _cols_dev(DS2MM, ctx, nm)
    if S.shape[0] != nd:
        raise ValueError("DipSource2MEGMat must have one column per dipole")
    out = torch.empty((nd, nm), dtype=torch.float64, device=_dev(ctx))
    check(ctx.lib.omg_gain_meg_dev(ctx.handle, N, _ptr(H), ld, packed, _ptr(D), nd, _ptr(Vc), nm, _ptr(S),
                                   _prec(precision), _ptr(out)))
    return out.T


def _cortical_domain(geom: Geometry, domain_name: str) -> int:
    if geom.domain_names is None or domain_name not in geom.domain_names:
        raise OMGError(-1, f"CorticalMat: unknown domain {domain_name!r}")   # Geometry::domain throws
    return geom.domain_names.index(domain_name)


def CorticalMat(geom: Geometry, M, domain_name: str = "CORTEX", alpha: float = -1.0, beta: float = -1.0,
                filename: str = "", integrator: Optional[Integrator] = None) -> torch.Tensor:
    """CorticalMat(geo, M, domain_name, alpha, beta, filename, integrator)
    (assembleHeadMat.cpp:168-236, om_assemble -CM): N x n_electrodes.  M is
    Head2EEGMat (dense, torch sparse or the sparse triple).  alpha < 0 picks
    alpha and beta automatically.  `filename` caches the null-space projector
    as the reference does: read from the file when it exists (.bin), else
    computed and written there."""
    from . import io
    import os
    ctx = geom.ctx
    N = geom.size
    dev = _dev(ctx)
    ne, r, c, v = _sparse_rows(M, ctx, N)
    dom = _cortical_domain(geom, domain_name)
    it = _default(integrator, 3, 0, 0.005)
    pin = pout = None
    if filename and os.path.exists(filename):
        P = torch.as_tensor(io.read_bin(filename)[1]).to(dev, torch.float64)
        if tuple(P.shape) != (N, N):
            raise OMGError(-6, f"CorticalMat: {filename} is not an {N} x {N} projector")
        pin = P.T.contiguous()
    elif filename:
        pout = torch.empty((N, N), dtype=torch.float64, device=dev)
    out = torch.empty((ne, N), dtype=torch.float64, device=dev)   # column-major N x ne
    check(ctx.lib.omg_corticalmat_dev(ctx.handle, geom.handle, ctypes.byref(it), dom, ne, r.numel(), _ptr(r),
                                      _ptr(c), _ptr(v), float(alpha), float(beta), _ptr(pin), _ptr(pout), _ptr(out)))
    if pout is not None:
        io.write_bin(filename, pout.T.cpu().numpy())
    return out.T


def CorticalMat2(geom: Geometry, M, domain_name: str = "CORTEX", gamma: float = 1.0, filename: str = "",
                 integrator: Optional[Integrator] = None) -> torch.Tensor:
    """CorticalMat2(geo, M, domain_name, gamma, filename, integrator)
    (assembleHeadMat.cpp:238-323, om_assemble -CM with one number):
    N x n_electrodes.  `filename` caches H (the head-matrix rows outside the
    cortex followed by M) as the reference does: its head-matrix rows are read
    from the file when it exists, else H is written there."""
    from . import io
    import os
    ctx = geom.ctx
    N = geom.size
    dev = _dev(ctx)
    ne, r, c, v = _sparse_rows(M, ctx, N)
    dom = _cortical_domain(geom, domain_name)
    it = _default(integrator, 3, 0, 0.005)
    nl = ctypes.c_int64()
    check(ctx.lib.omg_cortical_rows(geom.handle, dom, ctypes.byref(nl)))
    nl = nl.value
    rin = rout = None
    if filename and os.path.exists(filename):
        H = torch.as_tensor(io.read_bin(filename)[1])
        if tuple(H.shape) != (nl + ne, N):
            raise OMGError(-6, f"CorticalMat2: {filename} is not an {nl + ne} x {N} matrix")
        rin = H[:nl].to(dev, torch.float64).T.contiguous()       # column-major nl x N
    elif filename:
        rout = torch.empty((N, max(nl, 1)), dtype=torch.float64, device=dev)
    out = torch.empty((ne, N), dtype=torch.float64, device=dev)
    check(ctx.lib.omg_corticalmat2_dev(ctx.handle, geom.handle, ctypes.byref(it), dom, ne, r.numel(), _ptr(r),
                                       _ptr(c), _ptr(v), float(gamma), _ptr(rin), _ptr(rout), _ptr(out)))
    if rout is not None:   # the reference saves H = [rows; M] (assembleHeadMat.cpp:273-279)
        Md = torch.zeros((ne, N), dtype=torch.float64, device=dev)
        Md.index_put_((r, c), v, accumulate=True)
        io.write_bin(filename, torch.cat([rout.T[:nl], Md]).cpu().numpy())
    return out.T


def GainEEGadjoint(geom: Geometry, dipoles, electrodes, precision=FP64):
    """GainEEGadjoint(geo, dipoles, HM, H2EM) (gain.h:78-89), HM/H2EM assembled here."""
    return forward_gain(geom, dipoles, electrodes=electrodes, precision=precision)[0]


def GainMEGadjoint(geom: Geometry, dipoles, squids, precision=FP64):
    """GainMEGadjoint(geo, dipoles, HM, H2MM, DS2MM) (gain.h:91-104)."""
    return forward_gain(geom, dipoles, squids=squids, precision=precision)[1]


def GainEEGMEGadjoint(geom: Geometry, dipoles, electrodes, squids, precision=FP64):
    """GainEEGMEGadjoint (gain.h:106-136): (EEG leadfield, MEG leadfield)."""
    ge, gm, _ = forward_gain(geom, dipoles, electrodes=electrodes, squids=squids, precision=precision)
    return ge, gm
