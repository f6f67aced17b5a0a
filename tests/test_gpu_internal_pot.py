"""Internal potentials against the reference: Surf2VolMat and
DipSource2InternalPotMat (each dipole in its own domain, and all dipoles
forced into one domain) at points in every layer of a 3-layer (inward
meshes) and a 4-layer (outward meshes) head, some of them in the air, which
the reference drops.  Compared with om_assemble -H2IPM / -DS2IPM
(tests/golden/internal_potentials.npz) at 1e-12 relative Frobenius, and with
the oracle at larger point counts."""
import numpy as np
import pytest

from conftest import golden, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tag,layers,inward", [("3l", 3, True), ("4l_out", 4, False)])
def test_internal_potentials_match_reference(cuda, tag, layers, inward):
    from openmeeg_gb300 import api, workloads
    d = golden("internal_potentials")
    w = workloads.small(1, layers=layers, inward=inward)
    geo = api.Geometry.from_head(w.head)
    pts = d[f"points_{tag}"]
    H = api.Surf2VolMat(geo, pts).cpu().numpy()
    assert H.shape == d[f"h2ipm_{tag}"].shape
    assert rel(H, d[f"h2ipm_{tag}"]) <= 1e-12
    P = api.DipSource2InternalPotMat(geo, w.dipoles, pts).cpu().numpy()
    assert rel(P, d[f"ds2ipm_{tag}"]) <= 1e-12
    F = api.DipSource2InternalPotMat(geo, w.dipoles, pts, str(d[f"forced_{tag}"])).cpu().numpy()
    assert rel(F, d[f"ds2ipm_forced_{tag}"]) <= 1e-12


def test_surf2volmat_many_points_match_oracle(cuda):
    """5000 points spread over all layers and the air of an ico2 head (two
    chunks of the per-point scratch, which holds 4096 points), against the
    oracle."""
    from oracle import oracle
    from openmeeg_gb300 import api, workloads
    w = workloads.small(2, layers=3)
    geo = api.Geometry.from_head(w.head)
    rng = np.random.default_rng(5)
    u = rng.standard_normal((5000, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    pts = u * rng.uniform(0.0, 1.15, 5000)[:, None]
    H = api.Surf2VolMat(geo, pts).cpu().numpy()
    g = oracle.digest(w.head)
    R = oracle.surf2volmat(g, pts)
    assert H.shape == R.shape and 0 < H.shape[0] < 5000
    assert rel(H, R) <= 1e-12
    P = api.DipSource2InternalPotMat(geo, w.dipoles, pts).cpu().numpy()
    assert rel(P, oracle.dipsource2internalpotmat(g, w.dipoles, pts)) <= 1e-12


def test_all_points_dropped_and_empty_inputs(cuda):
    from openmeeg_gb300 import api, workloads
    w = workloads.small(1, layers=3)
    geo = api.Geometry.from_head(w.head)
    air = np.array([[0.0, 0.0, 1.5], [2.0, 0.0, 0.0]])
    assert tuple(api.Surf2VolMat(geo, air).shape) == (0, geo.size)
    assert tuple(api.DipSource2InternalPotMat(geo, w.dipoles, air).shape) == (0, w.dipoles.shape[0])
    assert tuple(api.Surf2VolMat(geo, np.zeros((0, 3))).shape) == (0, geo.size)
