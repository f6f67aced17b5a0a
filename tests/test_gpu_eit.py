"""EITSourceMat against the reference: point electrodes and electrodes with
radii (injection triangles found by the reference's walk over neighbouring
scalp triangles) on a 3-layer, a 4-layer outward-oriented and a perturbed ico2
head, compared with om_assemble -EITSM (tests/golden/eit_sources.npz) at
1e-12 relative Frobenius; a larger head against the oracle."""
import numpy as np
import pytest

from conftest import golden, rel

pytestmark = pytest.mark.gpu

CASES = [("3l", dict(layers=3)), ("4l_out", dict(layers=4, inward=False)),
         ("ico2_pert", dict(subdiv=2, layers=3, perturb=True))]


@pytest.mark.parametrize("tag,kw", CASES)
def test_eit_source_matches_reference(cuda, tag, kw):
    from openmeeg_gb300 import api, workloads
    d = golden("eit_sources")
    w = workloads.small(**{"subdiv": 1, **kw})
    geo = api.Geometry.from_head(w.head)
    el = d[f"electrodes_{tag}"]
    A = api.EITSourceMat(geo, el[:, :3]).cpu().numpy()
    assert A.shape == d[f"eit_points_{tag}"].shape
    assert rel(A, d[f"eit_points_{tag}"]) <= 1e-12
    B = api.EITSourceMat(geo, el).cpu().numpy()
    assert rel(B, d[f"eit_radii_{tag}"]) <= 1e-12


def test_eit_source_config0_head_matches_oracle(cuda):
    """config0's ico3 head, 64 electrodes with radii up to 0.2 (several scalp
    triangles each), against the oracle."""
    from oracle import oracle
    from openmeeg_gb300 import api, workloads
    w = workloads.config0()
    geo = api.Geometry.from_head(w.head)
    rng = np.random.default_rng(11)
    el = np.hstack([w.electrodes[:, :3], rng.choice([0.0, 0.05, 0.1, 0.2], size=(w.electrodes.shape[0], 1))])
    A = api.EITSourceMat(geo, el).cpu().numpy()
    g = oracle.digest(w.head)
    R = oracle.eitsourcemat(g, el)
    assert max(len(x) for x in oracle.injection_triangles(g, el)) > 3
    assert rel(A, R) <= 1e-12
