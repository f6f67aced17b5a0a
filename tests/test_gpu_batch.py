"""Batched forward (one captured CUDA graph over many head models).

Each model's gains must equal the single-model forward_gain of the same
precision: the batch enqueues the same kernels with the same inputs, so the
tolerance is 1e-12 (relative Frobenius).  Also: replays are reproducible,
new dipoles and new conductivities give the single-model answers, a dipole
outside the planned domains is reported, and the branch autotuner runs.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    import torch
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


@pytest.fixture(scope="module")
def heads(cuda):
    from openmeeg_gb300 import api, workloads
    ws = workloads.batch_small()
    return ws, [api.Geometry.from_head(w.head) for w in ws]


def _single(geo, w, dip, prec):
    from openmeeg_gb300 import api
    sq = w.squids if len(w.squids) else None
    ge, gm, _ = api.forward_gain(geo, dip, w.electrodes, sq, precision=prec)
    return ge, gm


def _batch(ws, geos, prec, nb):
    from openmeeg_gb300 import api
    return api.BatchForward([(g, w.dipoles, w.electrodes, w.squids) for g, w in zip(geos, ws)], precision=prec,
                            n_branches=nb)


@pytest.mark.parametrize("prec,nb", [("fp64", 3), ("mixed", 2)])
def test_batch_matches_single_model_path(heads, prec, nb):
    ws, geos = heads
    b = _batch(ws, geos, prec, nb)
    assert b.info()["n_branches"] == nb
    b.run()
    for i, (w, g) in enumerate(zip(ws, geos)):
        ge, gm = b.gains(i)
        re, rm = _single(g, w, w.dipoles, prec)
        assert _rel(ge, re) <= 1e-12, i
        if rm is not None:
            assert _rel(gm, rm) <= 1e-12, i
        else:
            assert gm is None


def test_batch_mixed_close_to_fp64(heads):
    ws, geos = heads
    b = _batch(ws, geos, "mixed", 4)
    b.run()
    for i, (w, g) in enumerate(zip(ws, geos)):
        ge, gm = b.gains(i)
        re, rm = _single(g, w, w.dipoles, "fp64")
        assert _rel(ge, re) <= 1e-6, i
        if rm is not None:
            assert _rel(gm, rm) <= 1e-6, i


def test_batch_replay_is_reproducible_and_takes_new_dipoles(heads):
    import torch
    from openmeeg_gb300 import synthetic as syn
    ws, geos = heads
    b = _batch(ws, geos, "mixed", 2)
    b.run()
    first = [b.gains(i) for i in range(len(ws))]
    b.run()
    for i in range(len(ws)):
        ge, gm = b.gains(i)
        assert torch.equal(ge, first[i][0])
    new = syn.random_dipoles(ws[1].dipoles.shape[0], 991, rmax=0.7)
    b.set_dipoles(1, new)
    b.run()
    ge, _ = b.gains(1)
    re, _ = _single(geos[1], ws[1], new, "mixed")
    assert _rel(ge, re) <= 1e-12


def test_batch_reports_dipole_outside_planned_domains(heads):
    from openmeeg_gb300 import OMGError
    ws, geos = heads
    b = _batch(ws, geos, "fp64", 2)
    b.run()
    bad = ws[0].dipoles.copy()
    bad[0, :3] = [0.0, 0.0, 0.895]           # inside the skull layer (0.87 < r < 0.92)
    b.set_dipoles(0, bad)
    with pytest.raises(OMGError) as e:
        b.run()
    assert "not planned" in str(e.value)
    b.set_dipoles(0, ws[0].dipoles)          # the batch stays usable
    b.run()
    ge, _ = b.gains(0)
    re, _ = _single(geos[0], ws[0], ws[0].dipoles, "fp64")
    assert _rel(ge, re) <= 1e-12


def test_batch_follows_conductivity_changes(cuda):
    from openmeeg_gb300 import api, workloads
    ws = workloads.batch_small()[:2]
    geos = [api.Geometry.from_head(w.head) for w in ws]
    b = _batch(ws, geos, "mixed", 2)
    b.run()
    sig = [d[2] for d in ws[0].head.domains]
    new = [s * 1.3 if s > 0 else 0.0 for s in sig]
    geos[0].set_conductivities(new)
    b.run()
    ge, _ = b.gains(0)
    re, _ = _single(geos[0], ws[0], ws[0].dipoles, "mixed")
    assert _rel(ge, re) <= 1e-12


def test_batch_autotune_and_info(heads, tmp_path, monkeypatch):
    ws, geos = heads
    monkeypatch.setenv("OMG_TUNE_CACHE", str(tmp_path / "tune.txt"))
    b = _batch(ws, geos, "mixed", 0)
    inf = b.info()
    assert inf["n_branches"] in (1, 2, 4) and inf["tuned_ms"] > 0
    assert inf["launches_per_run"] > 100 and inf["graph_nodes"] >= inf["launches_per_run"]
    assert "batch_branches" in (tmp_path / "tune.txt").read_text()
    b2 = _batch(ws, geos, "mixed", 0)     # cached choice: no timing pass
    assert b2.info()["n_branches"] == inf["n_branches"] and b2.info()["tuned_ms"] == 0
    b2.run()
    for i, (w, g) in enumerate(zip(ws, geos)):
        ge, _ = b2.gains(i)
        re, _ = _single(g, w, w.dipoles, "mixed")
        assert _rel(ge, re) <= 1e-12


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_batch_of_shared_vertex_heads(cuda, tmp_path, prec):
    """HeadNNa1 (hemispheres sharing the vertices of their cut mesh) in a batch
    beside a nested head: assembled on the vertex copies and folded, as the
    single-model path does; each model's gains equal the single-model ones."""
    from conftest import golden
    from openmeeg_gb300 import api, workloads
    R = golden("reference_heads")
    for fn, tx in zip(R["HeadNNa1_files"], R["HeadNNa1_texts"]):
        (tmp_path / str(fn)).write_text(str(tx))
    f = [str(x) for x in R["HeadNNa1_files"]]
    g1 = api.Geometry(str(tmp_path / f[0]), str(tmp_path / f[1]))
    w2 = workloads.small(1, layers=3)
    g2 = api.Geometry.from_head(w2.head)
    models = [(g1, R["HeadNNa1_dipoles"], R["HeadNNa1_electrodes"], R["HeadNNa1_squids"]),
              (g2, w2.dipoles, w2.electrodes, w2.squids)]
    b = api.BatchForward(models, precision=prec, n_branches=2)
    b.run()
    for i, (g, dip, el, sq) in enumerate(models):
        ge, gm = b.gains(i)
        re, rm, _ = api.forward_gain(g, dip, el, sq, precision=prec)
        assert _rel(ge, re) <= 1e-12 and _rel(gm, rm) <= 1e-12, i
