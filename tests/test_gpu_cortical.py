"""Cortical mapping on the GPU (omg_corticalmat_dev / omg_corticalmat2_dev,
api.CorticalMat / CorticalMat2) against the reference's own om_assemble -CM
outputs (tests/golden/cortical.npz, made by tests/golden/make_golden.py), and
the pivoted FP64 LU behind them.

The library solves one symmetric indefinite KKT system by LU with partial
pivoting where the reference uses an SVD pseudo-inverse (CorticalMat) or two
inverses (CorticalMat2); the forms agree to the conditioning of the problem:
relative Frobenius 1e-9 on the small heads, 1e-8 on config0's column norms and
random projections."""
import ctypes

import numpy as np
import pytest

from conftest import golden, rel

pytestmark = pytest.mark.gpu


def _lu_hook():
    from openmeeg_gb300 import _lib
    f = _lib.load().omg_internal_lu_solve
    f.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


@pytest.mark.parametrize("n", [5, 300, 1000, 4100])
def test_lu_partial_pivoting_solve(cuda, n):
    """Random nonsymmetric systems whose leading entries are zero (no LU
    without row exchanges), across several 64-column panels."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(n)
    A = torch.randn(n, n, device="cuda", dtype=torch.float64, generator=g)
    A[: n // 2, : n // 2] *= 1e-3
    A[0, 0] = 0.0
    X = torch.randn(n, 7, device="cuda", dtype=torch.float64, generator=g)
    B = A @ X
    Ac, Bc = A.T.contiguous(), B.T.contiguous()      # column-major
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert _lu_hook()(n, 7, p(Ac), p(Bc), p(err)) == 0 and int(err.item()) == 0
    res = torch.linalg.norm(A @ Bc.T - B) / (torch.linalg.norm(A) * torch.linalg.norm(Bc))
    assert float(res) < 1e-14, float(res)


def test_lu_reports_an_exactly_singular_matrix(cuda):
    import torch
    from openmeeg_gb300 import _lib
    n = 200
    A = torch.randn(n, n, device="cuda", dtype=torch.float64)
    A[:, 37] = 0.0
    B = torch.randn(n, 1, device="cuda", dtype=torch.float64)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    _lu_hook()(n, 1, p(A), p(B), p(err))
    assert int(err.item()) == -9 and _lib.ERRORS[-9] == "OMG_ERR_SINGULAR"


def _head1(tmp_path):
    from openmeeg_gb300 import api, io
    G = golden("cortical")
    for fn, tx in zip(G["head1_files"], G["head1_texts"]):
        (tmp_path / str(fn)).write_text(str(tx))
    geo = api.Geometry(str(tmp_path / "Head1.geom"), str(tmp_path / "Head1.cond"))
    return geo, io.read_sensors_txt(str(tmp_path / "Head1.patches"))[1]


def _small():
    from openmeeg_gb300 import api, workloads
    w = workloads.small(1, layers=3)
    return api.Geometry.from_meshes(w.head.vertices, w.head.triangles, w.head.domains), w.electrodes


@pytest.mark.parametrize("tag,args", [("auto", ()), ("ab", (1e-4, 1.58e-2))])
def test_corticalmat_head1_matches_reference(cuda, tmp_path, tag, args):
    from openmeeg_gb300 import api
    geo, el = _head1(tmp_path)
    M = api.Head2EEGMat(geo, el)
    X = api.CorticalMat(geo, M, "Brain", *args).cpu().numpy()
    assert rel(X, golden("cortical")[f"head1_{tag}"]) < 1e-9


@pytest.mark.parametrize("tag", ["auto", "ab", "gamma"])
def test_corticalmat_small_head_matches_reference(cuda, tag):
    from openmeeg_gb300 import api
    geo, el = _small()
    M = api.Head2EEGMat(geo, el, sparse=True)
    if tag == "gamma":
        X = api.CorticalMat2(geo, M, "Brain", 12.4)
    else:
        X = api.CorticalMat(geo, M, "Brain", *(() if tag == "auto" else (1e-4, 1.58e-2)))
    assert rel(X.cpu().numpy(), golden("cortical")[f"ico1_3l_{tag}"]) < 1e-9


@pytest.mark.parametrize("tag", ["auto", "ab", "gamma"])
def test_corticalmat_config0_matches_reference(cuda, tag):
    """N = 4486, 64 electrodes: the reference's column norms and its projection
    on a seeded random vector (the fixture keeps those, not the whole matrix)."""
    import sys
    from conftest import ROOT
    sys.path.insert(0, str(ROOT) + "/tests/golden")
    from make_golden import cortical_probe
    from openmeeg_gb300 import api, workloads
    w = workloads.config0()
    geo = api.Geometry.from_meshes(w.head.vertices, w.head.triangles, w.head.domains)
    M = api.Head2EEGMat(geo, w.electrodes, sparse=True)
    X = (api.CorticalMat2(geo, M, "Brain", 12.4) if tag == "gamma" else
         api.CorticalMat(geo, M, "Brain", *(() if tag == "auto" else (1e-4, 1.58e-2)))).cpu().numpy()
    G = golden("cortical")
    assert rel(np.linalg.norm(X, axis=0), G[f"config0_{tag}_norms"]) < 1e-8
    assert rel(X.T @ cortical_probe(w.head), G[f"config0_{tag}_proj"]) < 1e-8


def test_cortical_cache_files(cuda, tmp_path):
    """The reference's cache files: CorticalMat writes the null-space projector P
    when the file is missing and uses it when present; CorticalMat2 writes
    H = [head-matrix rows outside the cortex; M] and reads its rows back."""
    from openmeeg_gb300 import api, io
    geo, el = _small()
    M = api.Head2EEGMat(geo, el)
    f1 = str(tmp_path / "P.bin")
    X1 = api.CorticalMat(geo, M, "Brain", 1e-4, 1.58e-2, f1).cpu().numpy()
    P = io.read_bin(f1)[1]
    assert np.abs(P - P.T).max() < 1e-12 and np.abs(P @ P - P).max() < 1e-10
    X2 = api.CorticalMat(geo, M, "Brain", 1e-4, 1.58e-2, f1).cpu().numpy()
    assert rel(X2, X1) < 1e-9 and rel(X2, golden("cortical")["ico1_3l_ab"]) < 1e-9
    f2 = str(tmp_path / "H.bin")
    Y1 = api.CorticalMat2(geo, M, "Brain", 12.4, f2).cpu().numpy()
    H = io.read_bin(f2)[1]
    assert H.shape == (286 - 42 - 80 + 16, 286)
    assert np.array_equal(H[-16:], M.cpu().numpy())
    Y2 = api.CorticalMat2(geo, M, "Brain", 12.4, f2).cpu().numpy()
    assert rel(Y2, Y1) < 1e-12


def test_cortical_domain_checks(cuda):
    """assembleHeadMat.cpp:182-183: the source domain must be bounded by one
    interface of one mesh (Skull has two); unknown domains are refused."""
    from openmeeg_gb300 import api
    from openmeeg_gb300._lib import OMGError
    geo, el = _small()
    M = api.Head2EEGMat(geo, el)
    for name in ("Skull", "Nowhere"):
        with pytest.raises(OMGError):
            api.CorticalMat(geo, M, name)
