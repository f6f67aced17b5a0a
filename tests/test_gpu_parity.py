"""GPU parity of the CUDA forward path against the reference's own outputs
(golden fixtures made by tests/golden/make_golden.py) and the CPU oracle.

Tolerances: FP64 path -- relative Frobenius 1e-12 for assembled matrices,
1e-10 for gains (the reference's parity target); mixed precision -- 1e-6 on
gains against the FP64 result.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden, rel

pytestmark = pytest.mark.gpu

TOL_MAT = 1e-12
TOL_GAIN = 1e-10
TOL_MIXED = 1e-6


def _api():
    from openmeeg_gb300 import api
    return api


def _w(name):
    from openmeeg_gb300 import workloads
    return {
        "small_ico1_3l": lambda: workloads.small(1, layers=3),
        "small_ico1_4l_out": lambda: workloads.small(1, layers=4, inward=False),
        "small_ico2_3l_pert": lambda: workloads.small(2, layers=3, perturb=True),
        "config0": lambda: workloads.config0(),
    }[name]()


@pytest.mark.parametrize("name", ["small_ico1_3l", "small_ico1_4l_out"])
def test_headmat_matches_reference(cuda, name):
    from openmeeg_gb300 import io
    api = _api()
    G = golden(name)
    w = _w(name)
    geo = api.Geometry.from_head(w.head)
    HM = api.HeadMat(geo).cpu().numpy()
    N = HM.shape[0]
    ref = io.unpack_upper(G["hm_packed"], N)
    assert rel(HM, ref) < TOL_MAT
    assert np.array_equal(HM, HM.T)
    packed = api.HeadMatPacked(geo).cpu().numpy()
    assert np.array_equal(packed, io.packed_upper(HM))


@pytest.mark.parametrize("name", ["small_ico1_3l", "small_ico1_4l_out", "small_ico2_3l_pert"])
def test_sources_and_sensors_match_reference(cuda, name):
    api = _api()
    G = golden(name)
    w = _w(name)
    geo = api.Geometry.from_head(w.head)
    assert rel(api.DipSourceMat(geo, w.dipoles).cpu().numpy(), G["dsm"]) < TOL_MAT
    assert rel(api.Head2EEGMat(geo, w.electrodes).cpu().numpy(), G["h2em"]) < TOL_MAT
    if "h2mm" in G:
        assert rel(api.Head2MEGMat(geo, w.squids).cpu().numpy(), G["h2mm"]) < 1e-11
    assert rel(api.DipSource2MEGMat(w.dipoles, w.squids).cpu().numpy(), G["ds2mm"]) < TOL_MAT


@pytest.mark.parametrize("name", ["small_ico1_3l", "small_ico1_4l_out", "small_ico2_3l_pert", "config0"])
def test_fp64_gain_matches_reference(cuda, name):
    api = _api()
    G = golden(name)
    w = _w(name)
    geo = api.Geometry.from_head(w.head)
    ge, gm, st = api.forward_gain(geo, w.dipoles, w.electrodes, w.squids, precision="fp64")
    assert rel(ge.cpu().numpy(), G["eeg"]) < TOL_GAIN
    assert rel(gm.cpu().numpy(), G["meg"]) < TOL_GAIN


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "config1_200.npz")), reason="config1 fixture absent")
def test_fp64_gain_config1_matches_reference(cuda):
    from openmeeg_gb300 import workloads
    api = _api()
    G = golden("config1_200")
    w = workloads.config1(200)
    geo = api.Geometry.from_head(w.head)
    ge, gm, _ = api.forward_gain(geo, w.dipoles, w.electrodes, w.squids, precision="fp64")
    assert rel(ge.cpu().numpy(), G["eeg"]) < TOL_GAIN
    assert rel(gm.cpu().numpy(), G["meg"]) < TOL_GAIN


def test_host_entry_point_equals_device_entry_point(cuda):
    api = _api()
    w = _w("small_ico1_3l")
    geo = api.Geometry.from_head(w.head)
    ge, gm, _ = api.forward_gain(geo, w.dipoles, w.electrodes, w.squids)
    he, hm, _ = api.forward_gain(geo, w.dipoles, w.electrodes, w.squids, host=True)
    assert np.array_equal(ge.cpu().numpy(), he) and np.array_equal(gm.cpu().numpy(), hm)
    # caller-provided outputs in pinned host memory (the copies go straight to them)
    import torch
    nd, ne, nm = len(w.dipoles), len(w.electrodes), len(w.squids)
    oe = torch.full((nd, ne), np.nan, dtype=torch.float64, pin_memory=True).numpy()
    om = torch.full((nd, nm), np.nan, dtype=torch.float64, pin_memory=True).numpy()
    pe, pm, _ = api.forward_gain(geo, w.dipoles, w.electrodes, w.squids, host=True, out=(oe, om))
    assert np.array_equal(pe, he) and np.array_equal(pm, hm) and np.array_equal(oe.T, he)
    with pytest.raises(ValueError):
        api.forward_gain(geo, w.dipoles, w.electrodes, w.squids, host=True, out=(oe[:, :-1], om))


@pytest.mark.parametrize("name", ["small_ico2_3l_pert", "config0"])
def test_mixed_gain_within_tolerance(cuda, name):
    api = _api()
    w = _w(name)
    geo = api.Geometry.from_head(w.head)
    ge, gm, _ = api.forward_gain(geo, w.dipoles, w.electrodes, w.squids, precision="fp64")
    xe, xm, st = api.forward_gain(geo, w.dipoles, w.electrodes, w.squids, precision="mixed")
    assert rel(xe.cpu().numpy(), ge.cpu().numpy()) < TOL_MIXED
    assert rel(xm.cpu().numpy(), gm.cpu().numpy()) < TOL_MIXED
    assert st["refinement_steps"] >= 1


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solver_matches_dense_solve(cuda, precision):
    api = _api()
    w = _w("small_ico2_3l_pert")
    geo = api.Geometry.from_head(w.head)
    HM = api.HeadMat(geo).cpu().numpy()
    rng = np.random.default_rng(0)
    B = rng.standard_normal((HM.shape[0], 5))
    X = api.Solver(geo, precision=precision).solve(B).cpu().numpy()
    ref = np.linalg.solve(HM, B)
    if precision == "fp64":
        assert rel(X, ref) < 1e-11
    else:
        # the mixed solver refines against its own (mixed-assembled) head matrix until the predicted
        # error (last correction times the contraction factor) is below its tolerance, 1e-6
        Hm = api.HeadMat(geo, precision="mixed").cpu().numpy()
        assert rel(X, np.linalg.solve(Hm, B)) < 1e-7
        assert rel(X, ref) < 1e-6
    # factoring a caller-provided HeadMat gives the same solution
    X2 = api.Solver(geo, precision="fp64", hm=HM).solve(B).cpu().numpy()
    assert rel(X2, ref) < 1e-11


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solver_pivots_when_the_matrix_is_not_quasi_definite(cuda, precision):
    """A head matrix whose triangle block has a diagonal entry of the wrong sign
    is no longer quasi-definite: the LDL^T without pivoting stops there
    (OMG_ERR_NOT_DEFINITE) and the solver refactors the matrix by the FP64 LU
    with partial pivoting, which solves any nonsingular matrix as the
    reference's Bunch-Kaufman does; an exactly singular one is reported."""
    from openmeeg_gb300._lib import OMGError
    api = _api()
    w = _w("small_ico1_3l")
    geo = api.Geometry.from_head(w.head)
    HM = api.HeadMat(geo).cpu().numpy()
    nv = sum(v.shape[0] for v in w.head.vertices)   # reference numbering: vertices, then triangles
    A = HM.copy()
    A[nv + 5, nv + 5] = -10.0 * abs(A[nv + 5, nv + 5])
    B = np.random.default_rng(1).standard_normal((A.shape[0], 3))
    X = api.Solver(geo, precision=precision, hm=A).solve(B).cpu().numpy()
    assert rel(X, np.linalg.solve(A, B)) < 1e-10
    A[:, nv + 7] = 0.0
    A[nv + 7, :] = 0.0
    with pytest.raises(OMGError) as e:
        api.Solver(geo, precision=precision, hm=A)
    assert e.value.code == -9


def test_mixed_solver_falls_back_to_fp64_when_refinement_stalls(cuda):
    """An unreachable refinement tolerance: the mixed refinement stalls, the
    solver rebuilds its (mixed-assembled) head matrix and solves it in FP64."""
    api = _api()
    w = _w("small_ico2_3l_pert")
    geo = api.Geometry.from_head(w.head)
    Hm = api.HeadMat(geo, precision="mixed").cpu().numpy()
    B = np.random.default_rng(2).standard_normal((Hm.shape[0], 4))
    s = api.Solver(geo, precision="mixed")
    s.set_refinement(1e-300, 2)
    X = s.solve(B).cpu().numpy()
    assert rel(X, np.linalg.solve(Hm, B)) < 1e-11
    X2 = s.solve(B).cpu().numpy()           # the solver stays FP64 from then on
    assert rel(X2, X) < 1e-14


def test_headmat_config0_matches_oracle(cuda):
    from oracle import oracle
    api = _api()
    w = _w("config0")
    geo = api.Geometry.from_head(w.head)
    HM = api.HeadMat(geo).cpu().numpy()
    g = oracle.digest(w.head)
    ref = oracle.headmat(g)
    assert HM.shape == (4486, 4486)
    assert rel(HM, ref) < TOL_MAT


def test_geometry_file_loader(cuda, tmp_path):
    from oracle import ref_runner
    api = _api()
    w = _w("small_ico1_3l")
    ref_runner.write_head(str(tmp_path), w.head)
    g1 = api.Geometry(str(tmp_path / "head.geom"), str(tmp_path / "head.cond"))
    g2 = api.Geometry.from_head(w.head)
    assert g1.size == g2.size == 286
    assert rel(api.HeadMat(g1).cpu().numpy(), api.HeadMat(g2).cpu().numpy()) < 1e-15


def test_handles_can_be_destroyed_in_any_order(cuda):
    from openmeeg_gb300 import _lib
    import ctypes
    api = _api()
    w = _w("small_ico1_3l")
    ctx = api.Context(0)
    geo = api.Geometry.from_head(w.head, ctx)
    sv = api.Solver(geo)
    lib = _lib.load()
    # context first, then geometry, then solver: all three stay valid until the last goes
    assert lib.omg_context_destroy(ctx.handle) == 0
    ctx.handle = None
    x = sv.solve(np.ones(geo.size)).cpu().numpy()
    assert np.all(np.isfinite(x))
    assert lib.omg_geometry_destroy(geo.handle) == 0
    geo.handle = None
    x2 = sv.solve(np.ones(286)).cpu().numpy()
    assert np.array_equal(x, x2)
    assert lib.omg_solver_destroy(sv.handle) == 0
    sv.handle = None


def test_empty_and_invalid_inputs(cuda):
    api = _api()
    w = _w("small_ico1_3l")
    geo = api.Geometry.from_head(w.head)
    # no dipoles: empty gains
    ge, gm, _ = api.forward_gain(geo, np.zeros((0, 6)), w.electrodes, w.squids)
    assert ge.shape == (16, 0) and gm.shape == (10, 0)
    # EEG only / MEG only
    ge, gm, _ = api.forward_gain(geo, w.dipoles, w.electrodes, None)
    assert gm is None and ge.shape == (16, 8)
    # a dipole outside every domain is reported, not silently zeroed
    bad = w.dipoles.copy()
    bad[0, :3] = [5.0, 0.0, 0.0]   # outside the head: lies in "Air" (conductivity 0) -> zero column
    D = api.DipSourceMat(geo, bad).cpu().numpy()
    assert np.all(D[:, 0] == 0.0)
    # degenerate triangle
    V = [v.copy() for v in w.head.vertices]
    T = [t.copy() for t in w.head.triangles]
    T[0][0] = [0, 0, 1]
    with pytest.raises(api.OMGError):
        api.Geometry.from_meshes(V, T, w.head.domains)
    # open mesh (one triangle removed)
    T = [t.copy() for t in w.head.triangles]
    T[1] = T[1][1:]
    with pytest.raises(api.OMGError):
        api.Geometry.from_meshes(V, T, w.head.domains)


@pytest.mark.parametrize("name", ["small_ico2_3l_pert", "config0"])
def test_mixed_headmat_close_to_fp64(cuda, name):
    """Far pairs by the FP32 product rule, near pairs in FP64: the assembled
    matrix stays within 1e-6 (relative Frobenius) of the FP64 drop-in."""
    api = _api()
    w = _w(name)
    geo = api.Geometry.from_head(w.head)
    H64 = api.HeadMat(geo, precision="fp64").cpu().numpy()
    H32 = api.HeadMat(geo, precision="mixed").cpu().numpy()
    assert np.array_equal(H32, H32.T)
    assert rel(H32, H64) < 1e-6
