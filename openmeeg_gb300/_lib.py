"""ctypes binding of libomg_gb300.so (the C ABI declared in include/openmeeg_gb300.h).

Loading fails loudly when the library is missing or cannot be loaded: there
is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libomg_gb300.so")

OMG_OK = 0
ERRORS = {
    -1: "OMG_ERR_INVALID", -2: "OMG_ERR_CUDA", -3: "OMG_ERR_NOT_DEFINITE", -4: "OMG_ERR_NOT_CONVERGED",
    -5: "OMG_ERR_NOMEM", -6: "OMG_ERR_IO", -7: "OMG_ERR_UNSUPPORTED", -8: "OMG_ERR_TIMEOUT", -9: "OMG_ERR_SINGULAR",
}
PREC_FP64 = 0
PREC_MIXED = 1

c_i32, c_i64, c_dbl, c_vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p
P_i64 = ctypes.POINTER(ctypes.c_int64)
P_i32 = ctypes.POINTER(ctypes.c_int32)
P_dbl = ctypes.POINTER(ctypes.c_double)


class OMGError(RuntimeError):
    """Raised for a non-zero status of the C ABI; `.code` holds the status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Integrator(ctypes.Structure):
    """Integrator(order, levels, tol) (OpenMEEG/include/integrator.h:192-196)."""
    _fields_ = [("order", ctypes.c_int32), ("levels", ctypes.c_int32), ("tol", ctypes.c_double)]

    def __init__(self, order=3, levels=0, tol=0.0001):
        super().__init__(int(order), int(levels), float(tol))

    def __repr__(self):
        return f"Integrator({self.order},{self.levels},{self.tol})"


class GeometryInfo(ctypes.Structure):
    _fields_ = [("n_vertices", c_i64), ("n_triangles", c_i64), ("n_unknowns", c_i64),
                ("n_triangle_unknowns", c_i64), ("n_meshes", c_i32), ("n_domains", c_i32),
                ("n_mesh_pairs", c_i32), ("nested", c_i32)]


class MeshLayout(ctypes.Structure):
    _fields_ = [("vbeg", c_i64), ("vend", c_i64), ("tri_unknown", c_i64), ("n_triangles", c_i64), ("barrier", c_i32),
                ("orientation", c_i32), ("outermost", c_i32), ("reserved", c_i32)]


class MeshPair(ctypes.Structure):
    _fields_ = [("m1", c_i32), ("m2", c_i32), ("orientation", c_i32), ("reserved", c_i32), ("cS", c_dbl),
                ("cN", c_dbl), ("cD", c_dbl)]


class GainStats(ctypes.Structure):
    _fields_ = [("t_total_ms", c_dbl), ("t_headmat_ms", c_dbl), ("t_sources_ms", c_dbl), ("t_factor_ms", c_dbl),
                ("t_solve_ms", c_dbl), ("refinement_steps", c_i32), ("residual_mode", c_i32),
                ("final_residual", c_dbl), ("device_bytes", c_i64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchModel(ctypes.Structure):
    _fields_ = [("geometry", c_vp), ("dipoles", P_dbl), ("n_dipoles", c_i64), ("electrodes", P_dbl),
                ("n_electrodes", c_i64), ("squids", P_dbl), ("n_squids", c_i64)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("n_models", c_i32), ("n_branches", c_i32), ("precision", c_i32), ("max_refine_steps", c_i32),
                ("launches_per_run", c_i64), ("graph_nodes", c_i64), ("graph_bytes_estimate", c_i64),
                ("tuned_ms", c_dbl)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# (name, restype, argtypes)
_PROTOS = [
    ("omg_last_error", ctypes.c_char_p, []),
    ("omg_version", ctypes.c_char_p, []),
    ("omg_context_create", c_i32, [ctypes.c_int, ctypes.POINTER(c_vp)]),
    ("omg_context_destroy", c_i32, [c_vp]),
    ("omg_context_set_stream", c_i32, [c_vp, c_vp]),
    ("omg_context_synchronize", c_i32, [c_vp]),
    ("omg_context_kernel_launches", c_i64, [c_vp]),
    ("omg_profile_enable", c_i32, [c_i32]),
    ("omg_profile_read", c_i32, [c_i32, ctypes.c_char_p, P_i64, P_dbl, P_i32]),
    ("omg_geometry_create", c_i32, [c_vp, c_i32, P_i64, P_dbl, P_i64, P_i64, c_i32, P_i32, P_i32, P_dbl,
                                    ctypes.POINTER(c_vp)]),
    ("omg_geometry_load", c_i32, [c_vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(c_vp)]),
    ("omg_geometry_destroy", c_i32, [c_vp]),
    ("omg_geometry_get_info", c_i32, [c_vp, ctypes.POINTER(GeometryInfo)]),
    ("omg_geometry_set_conductivities", c_i32, [c_vp, P_dbl]),
    ("omg_headmat_dev", c_i32, [c_vp, c_vp, ctypes.POINTER(Integrator), c_i32, c_vp, c_i64]),
    ("omg_headmat_packed_dev", c_i32, [c_vp, c_vp, ctypes.POINTER(Integrator), c_vp]),
    ("omg_dipsourcemat_dev", c_i32, [c_vp, c_vp, c_vp, c_i64, ctypes.POINTER(Integrator), c_i32, c_vp]),
    ("omg_head2eegmat_dev", c_i32, [c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp]),
    ("omg_head2megmat_dev", c_i32, [c_vp, c_vp, c_vp, c_i64, c_vp]),
    ("omg_head2megmat_noalloc_dev", c_i32, [c_vp, c_vp, c_vp, c_i64, c_vp]),
    ("omg_gain_eeg_dev", c_i32, [c_vp, c_i64, c_vp, c_i64, c_i32, c_vp, c_i64, c_i64, c_i64, c_vp, c_vp, c_vp, c_i32,
                                 c_vp]),
    ("omg_gain_meg_dev", c_i32, [c_vp, c_i64, c_vp, c_i64, c_i32, c_vp, c_i64, c_vp, c_i64, c_vp, c_i32, c_vp]),
    ("omg_corticalmat_dev", c_i32, [c_vp, c_vp, ctypes.POINTER(Integrator), c_i32, c_i64, c_i64, c_vp, c_vp, c_vp,
                                    ctypes.c_double, ctypes.c_double, c_vp, c_vp, c_vp]),
    ("omg_corticalmat2_dev", c_i32, [c_vp, c_vp, ctypes.POINTER(Integrator), c_i32, c_i64, c_i64, c_vp, c_vp, c_vp,
                                     ctypes.c_double, c_vp, c_vp, c_vp]),
    ("omg_cortical_rows", c_i32, [c_vp, c_i32, P_i64]),
    ("omg_dipsource2megmat_dev", c_i32, [c_vp, c_vp, c_i64, c_vp, c_i64, c_vp]),
    ("omg_geometry_get_layout", c_i32, [c_vp, c_i32, ctypes.POINTER(MeshLayout)]),
    ("omg_geometry_get_pairs", c_i32, [c_vp, c_i32, ctypes.POINTER(MeshPair), P_i32]),
    ("omg_dipole_domains_dev", c_i32, [c_vp, c_vp, c_vp, c_i64, c_vp]),
    ("omg_head2megmat_mesh_dev", c_i32, [c_vp, c_vp, c_vp, c_i64, c_i32, c_vp]),
    ("omg_dipsourcemat_vjp_dev", c_i32, [c_vp, c_vp, c_vp, c_i64, ctypes.POINTER(Integrator), c_i32, c_vp, c_i64,
                                         c_vp]),
    ("omg_gemm_f64_dev", c_i32, [c_vp, c_i32, c_i32, c_i64, c_i64, c_i64, c_dbl, c_vp, c_i64, c_vp, c_i64, c_dbl,
                                 c_vp, c_i64]),
    ("omg_solver_create", c_i32, [c_vp, c_vp, ctypes.POINTER(Integrator), c_i32, ctypes.POINTER(c_vp)]),
    ("omg_solver_from_headmat_dev", c_i32, [c_vp, c_vp, c_vp, c_i64, c_i32, ctypes.POINTER(c_vp)]),
    ("omg_solver_solve_dev", c_i32, [c_vp, c_vp, c_i64, c_i64]),
    ("omg_solver_set_refinement", c_i32, [c_vp, ctypes.c_double, c_i32]),
    ("omg_solver_destroy", c_i32, [c_vp]),
    ("omg_gain_dev", c_i32, [c_vp, c_vp, c_i32, ctypes.POINTER(Integrator), ctypes.POINTER(Integrator), c_vp, c_i64,
                             c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, ctypes.POINTER(GainStats)]),
    ("omg_gain_host", c_i32, [c_vp, c_vp, c_i32, ctypes.POINTER(Integrator), ctypes.POINTER(Integrator), P_dbl,
                              c_i64, P_dbl, c_i64, P_dbl, c_i64, P_dbl, P_dbl, ctypes.POINTER(GainStats)]),
    ("omg_surfsourcemat_dev", c_i32, [c_vp, c_vp, P_dbl, c_i64, P_i64, c_i64, ctypes.POINTER(Integrator), c_vp]),
    ("omg_surfsource2megmat_dev", c_i32, [c_vp, P_dbl, c_i64, P_i64, c_i64, c_vp, c_i64, c_vp]),
    ("omg_surf2volmat_dev", c_i32, [c_vp, c_vp, c_vp, c_i64, c_vp, P_i64]),
    ("omg_dipsource2internalpotmat_dev", c_i32, [c_vp, c_vp, c_vp, c_i64, c_vp, c_i64, c_i32, c_vp, P_i64]),
    ("omg_eitsourcemat_dev", c_i32, [c_vp, c_vp, c_vp, c_vp, c_i64, ctypes.POINTER(Integrator), c_vp]),
    ("omg_batch_create", c_i32, [c_vp, c_i32, ctypes.POINTER(BatchModel), c_i32, c_i32, ctypes.POINTER(c_vp)]),
    ("omg_batch_run", c_i32, [c_vp]),
    ("omg_batch_gain_dev", c_i32, [c_vp, c_i32, ctypes.POINTER(c_vp), ctypes.POINTER(c_vp)]),
    ("omg_batch_set_dipoles", c_i32, [c_vp, c_i32, P_dbl]),
    ("omg_batch_get_info", c_i32, [c_vp, ctypes.POINTER(BatchInfo)]),
    ("omg_batch_destroy", c_i32, [c_vp]),
]

EXPORTED = [p[0] for p in _PROTOS]

_lib = None
_lock = threading.Lock()


def load(path: str = LIB_PATH):
    """Load (once) and return the library with typed prototypes."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise OMGError(-2, f"CUDA library not built: {path} is missing (run __graft_entry__.build())")
            lib = ctypes.CDLL(path)
            for name, res, args in _PROTOS:
                f = getattr(lib, name)
                f.restype = res
                f.argtypes = args
            _lib = lib
    return _lib


def profile_enable(on: bool = True):
    check(load().omg_profile_enable(1 if on else 0))


def profile_read(max_entries: int = 64):
    """{kernel name: (launches, total ms)} recorded since the last read."""
    names = ctypes.create_string_buffer(32 * max_entries)
    launches = (ctypes.c_int64 * max_entries)()
    ms = (ctypes.c_double * max_entries)()
    n = ctypes.c_int32()
    check(load().omg_profile_read(max_entries, names, launches, ms, ctypes.byref(n)))
    out = {}
    for i in range(n.value):
        nm = names.raw[32 * i:32 * (i + 1)].split(b"\0", 1)[0].decode()
        out[nm] = (int(launches[i]), float(ms[i]))
    return out


def check(rc: int):
    if rc != OMG_OK:
        msg = load().omg_last_error().decode(errors="replace")
        raise OMGError(rc, msg)
    return rc
