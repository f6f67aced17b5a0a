"""The reference's own golden files for its Head1 test head
(tests/initialTest/Head1.*, MATLAB v7.3 / HDF5 written by its MatlabIO,
copied with their inputs into tests/golden/head1 by
tests/golden/make_golden.py): read by openmeeg_gb300.matio, and the oracle
pinned to them."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel

H1 = os.path.join(GOLDEN, "head1")


def mat(name):
    from openmeeg_gb300 import matio
    return matio.read_mat(os.path.join(H1, "Head1." + name))


def test_matio_reads_every_kind():
    """linop (Matrix), symmatrix (SymMatrix struct), MATLAB sparse."""
    expect = {"hm": ("sym", (286, 286)), "hm_inv": ("sym", (286, 286)), "dsm": ("full", (286, 6)),
              "h2em": ("sparse", (32, 286)), "h2mm": ("full", (162, 286)), "ds2mm": ("full", (162, 6)),
              "dgem": ("full", (32, 6)), "dgmm": ("full", (162, 6)), "ssm": ("full", (286, 42)),
              "sgem": ("full", (32, 42))}
    for name, (kind, shape) in expect.items():
        k, A = mat(name)
        assert k == kind and A.shape == shape, name
        assert np.isfinite(A).all()
    _, H = mat("hm")
    assert np.array_equal(H, H.T)
    _, E = mat("h2em")
    assert np.all((E != 0).sum(axis=1) <= 3) and np.allclose(E.sum(axis=1), 1.0)   # barycentric weights


def test_matio_rejects_other_files(tmp_path):
    from openmeeg_gb300 import io, matio
    p = tmp_path / "a.bin"
    io.write_bin(str(p), np.eye(3))
    with pytest.raises(ValueError):
        matio.read_mat(str(p))


def head1():
    from openmeeg_gb300 import io
    head = io.load_head(os.path.join(H1, "Head1.geom"), os.path.join(H1, "Head1.cond"))
    dip = io.read_matrix_txt(os.path.join(H1, "Head1.dip"))
    el = io.read_sensors_txt(os.path.join(H1, "Head1.patches"))[1]
    sq = io.read_sensors_txt(os.path.join(H1, "Head1.squids"))[1][:, :6]
    return head, dip, el, sq


def test_oracle_pinned_to_the_reference_head1_goldens():
    """The oracle against the matrices the reference's authors shipped: rounding
    level for the head matrix, its inverse, the sources, the sensors and the
    gains (1e-10 for H2MM, whose Ferguson sums cancel)."""
    from oracle import oracle
    head, dip, el, sq = head1()
    g = oracle.digest(head)
    HM = oracle.headmat(g)
    D = oracle.dsm(g, dip)
    E = oracle.h2em(g, el)
    M = oracle.h2mm(g, sq)
    S = oracle.ds2mm(dip, sq)
    assert rel(HM, mat("hm")[1]) < 1e-14
    assert rel(np.linalg.inv(HM), mat("hm_inv")[1]) < 1e-13
    assert rel(D, mat("dsm")[1]) < 1e-14
    assert np.array_equal(E, mat("h2em")[1])
    assert rel(M, mat("h2mm")[1]) < 1e-10
    assert rel(S, mat("ds2mm")[1]) < 1e-14
    assert rel(oracle.gain_eeg(HM, D, E), mat("dgem")[1]) < 1e-13
    assert rel(oracle.gain_meg(HM, D, M, S), mat("dgmm")[1]) < 1e-12
