"""The library (FP64 drop-in and mixed precision) against the reference's own
golden files for its Head1 test head (tests/initialTest/Head1.*, MATLAB v7.3,
read by openmeeg_gb300.matio from tests/golden/head1): the head matrix, the
sources and sensors, the adjoint gains, the direct-form gains from the
reference's own inverse, and SurfSourceMat of its source mesh.

Tolerances (relative Frobenius): 1e-12 for matrices, 1e-10 for H2MM (its
Ferguson sums cancel) and the FP64 gains, 1e-6 for the mixed gains."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel

pytestmark = pytest.mark.gpu

H1 = os.path.join(GOLDEN, "head1")


def mat(name):
    from openmeeg_gb300 import matio
    return matio.read_mat(os.path.join(H1, "Head1." + name))[1]


def inputs():
    from openmeeg_gb300 import api, io
    geo = api.Geometry(os.path.join(H1, "Head1.geom"), os.path.join(H1, "Head1.cond"))
    dip = io.read_matrix_txt(os.path.join(H1, "Head1.dip"))
    el = io.read_sensors_txt(os.path.join(H1, "Head1.patches"))[1]
    sq = io.read_sensors_txt(os.path.join(H1, "Head1.squids"))[1][:, :6]
    return geo, dip, el, sq


def test_head1_matrices_match_reference_goldens(cuda):
    from openmeeg_gb300 import api
    geo, dip, el, sq = inputs()
    np_ = lambda t: t.cpu().numpy()
    assert rel(np_(api.HeadMat(geo)), mat("hm")) < 1e-12
    assert rel(np_(api.DipSourceMat(geo, dip)), mat("dsm")) < 1e-12
    assert rel(np_(api.Head2EEGMat(geo, el)), mat("h2em")) < 1e-12
    assert rel(np_(api.Head2MEGMat(geo, sq)), mat("h2mm")) < 1e-10
    assert rel(np_(api.DipSource2MEGMat(dip, sq)), mat("ds2mm")) < 1e-12


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-6)])
def test_head1_gains_match_reference_goldens(cuda, precision, tol):
    from openmeeg_gb300 import api
    geo, dip, el, sq = inputs()
    ge, gm, _ = api.forward_gain(geo, dip, el, sq, precision=precision)
    assert rel(ge.cpu().numpy(), mat("dgem")) < tol
    assert rel(gm.cpu().numpy(), mat("dgmm")) < tol


def test_head1_direct_gains_from_the_reference_inverse(cuda):
    """om_gain -EEG / -MEG semantics with the reference's own HMinv, DSM and
    sensor matrices read from its .mat files."""
    from openmeeg_gb300 import api
    ge = api.GainEEG(mat("hm_inv"), mat("dsm"), mat("h2em")).cpu().numpy()
    gm = api.GainMEG(mat("hm_inv"), mat("dsm"), mat("h2mm"), mat("ds2mm")).cpu().numpy()
    assert rel(ge, mat("dgem")) < 1e-10
    assert rel(gm, mat("dgmm")) < 1e-10


def test_head1_surface_source_matches_reference_golden(cuda):
    from openmeeg_gb300 import api, io
    geo, _, _, _ = inputs()
    V, T = io.read_mesh(os.path.join(H1, "Head1.tri"))
    assert rel(api.SurfSourceMat(geo, V, T).cpu().numpy(), mat("ssm")) < 1e-10
