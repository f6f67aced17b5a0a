"""Cortical mapping oracle (oracle.corticalmat / corticalmat2, restating
OpenMEEG/src/assembleHeadMat.cpp:137-323) pinned to the reference's own
om_assemble -CM outputs (tests/golden/cortical.npz, made by
tests/golden/make_golden.py): the reference's Head1 with its patches, domain
and parameters (TestHead.cmake:94-96), and the seeded small_ico1_3l head."""
import numpy as np
import pytest

from conftest import golden, rel


def head1(tmp_path):
    from openmeeg_gb300 import io
    G = golden("cortical")
    for fn, tx in zip(G["head1_files"], G["head1_texts"]):
        (tmp_path / str(fn)).write_text(str(tx))
    head = io.load_head(str(tmp_path / "Head1.geom"), str(tmp_path / "Head1.cond"))
    electrodes = io.read_sensors_txt(str(tmp_path / "Head1.patches"))[1]
    return head, electrodes


@pytest.mark.parametrize("tag,args", [("auto", ()), ("ab", (1e-4, 1.58e-2))])
def test_oracle_corticalmat_head1_pinned_to_reference(tmp_path, tag, args):
    from oracle import oracle
    head, el = head1(tmp_path)
    g = oracle.digest(head)
    M = oracle.h2em(g, el)
    X, P = oracle.corticalmat(g, M, "Brain", *args)
    assert rel(X, golden("cortical")[f"head1_{tag}"]) < 1e-10
    # P: the orthogonal projector on the null space of the head-matrix rows outside the cortex
    mat, _ = oracle.headmatrix_rows(g, oracle.cortex_mesh(g, "Brain"))
    assert np.abs(P @ P - P).max() < 1e-12 and np.abs(mat @ P).max() < 1e-10 * np.abs(mat).max()


@pytest.mark.parametrize("tag", ["auto", "ab", "gamma"])
def test_oracle_corticalmat_small_head_pinned_to_reference(tag):
    from oracle import oracle
    from openmeeg_gb300 import workloads
    w = workloads.small(1, layers=3)
    g = oracle.digest(w.head)
    M = oracle.h2em(g, w.electrodes)
    if tag == "gamma":
        X, _ = oracle.corticalmat2(g, M, "Brain", 12.4)
    else:
        X, _ = oracle.corticalmat(g, M, "Brain", *(() if tag == "auto" else (1e-4, 1.58e-2)))
    assert rel(X, golden("cortical")[f"ico1_3l_{tag}"]) < 1e-10


def test_cortical_kkt_form_equals_the_reference_form():
    """The library solves [A mat^T; mat 0] [X; L] = [M^T; 0] (and the CorticalMat2
    system) instead of the reference's SVD pseudo-inverse / inverses; on the
    small head the two forms agree to rounding (numpy, both sides)."""
    from oracle import oracle
    from openmeeg_gb300 import workloads
    w = workloads.small(1, layers=3)
    g = oracle.digest(w.head)
    M = oracle.h2em(g, w.electrodes)
    mat, _ = oracle.headmatrix_rows(g, oracle.cortex_mesh(g, "Brain"))
    RR = oracle.gradient_norm2(g)
    nv, Nc, Nl, ne = g.V.shape[0], g.N, mat.shape[0], M.shape[0]
    d = np.full(Nc, 1.58e-2)
    d[:nv] = 1e-4
    A = M.T @ M + d[:, None] * RR
    K = np.zeros((Nc + Nl, Nc + Nl))
    K[:Nc, :Nc], K[Nc:, :Nc], K[:Nc, Nc:] = A, mat, mat.T
    rhs = np.zeros((Nc + Nl, ne))
    rhs[:Nc] = M.T
    X = np.linalg.solve(K, rhs)[:Nc]
    assert rel(X, oracle.corticalmat(g, M, "Brain", 1e-4, 1.58e-2)[0]) < 1e-10
