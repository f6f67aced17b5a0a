"""The BEM forward path against the analytic nested-sphere solutions, with
the reference test suite's tolerances for its sample head Head3
(tests/ComparisonTest_caller.cmake: EEG RDM and MAG < 0.03, MEG < 0.12 for
dipoles 1-5; dipole 6 is radial and its field vanishes).  The meshes, dipoles
and sensors are the reference's own (tests/golden/head3_analytic.npz); the
analytic values are those its suite ships, which the oracle's series
reproduces to 1e-12 (tests/test_cpu_oracle.py)."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _head3(cuda):
    from openmeeg_gb300 import api
    d = golden("head3_analytic")
    V = np.split(d["vertices"], np.cumsum(d["nverts"])[:-1])
    T = np.split(d["triangles"], np.cumsum(d["ntris"])[:-1])
    bounds = np.split(d["dom_bounds"], np.cumsum(d["dom_nb"])[:-1])
    domains = [(str(n), [int(b) for b in bd], float(s)) for n, bd, s in zip(d["dom_names"], bounds, d["dom_sigma"])]
    return d, api.Geometry.from_meshes(V, T, domains)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_head3_eeg_meg_match_analytic_series(cuda, prec):
    from oracle import analytic as an
    from openmeeg_gb300 import api
    d, geo = _head3(cuda)
    ge, gm, _ = api.forward_gain(geo, d["dipoles"], d["electrodes"], d["squids"][:, :6], precision=prec)
    ge = ge.cpu().numpy()
    gm = gm.cpu().numpy()
    r, m = an.rdm(ge, d["eeg_analytic"]), an.mag(ge, d["eeg_analytic"])
    assert r.max() < 0.03 and m.max() < 0.03, (r, m)
    r, m = an.rdm(gm[:, :5], d["meg_analytic"][:, :5]), an.mag(gm[:, :5], d["meg_analytic"][:, :5])
    assert r.max() < 0.12 and m.max() < 0.12, (r, m)
    assert np.abs(gm[:, 5]).max() < 1e-3 * np.abs(gm[:, :5]).max()
