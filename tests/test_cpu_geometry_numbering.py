"""The library's host-side geometry set-up (vertex copies, numbering, interface
orientation, barriers) on the reference's own heads, without a GPU: against
the oracle's restatement of Geometry::finalize (geometry.cpp) where it applies
(HeadMN1-3, HeadNNb1: barriers, an inverted interface, nested and non-nested
heads), and, on the heads whose interfaces are made of several meshes sharing
vertices (HeadNNa1, HeadNNc1), against the definition of the vertex copies
(geometry.h:100-108: equal coordinates are one vertex, numbered in order of
first appearance) and the size of the reference's own DipSourceMat."""
import ctypes

import numpy as np
import pytest

from conftest import golden


@pytest.fixture(scope="module")
def hook():
    from openmeeg_gb300 import build
    lib = ctypes.CDLL(build.build())
    f = lib.omg_internal_geometry_numbering
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char_p, ctypes.c_char_p] + [ctypes.c_void_p] * 6 + [ctypes.c_int64, ctypes.c_int64,
                                                                                 ctypes.c_int32]
    return f


@pytest.fixture(scope="module")
def ref():
    return golden("reference_heads")


def _files(ref, name, tmp_path):
    for fn, tx in zip(ref[f"{name}_files"], ref[f"{name}_texts"]):
        (tmp_path / str(fn)).write_text(str(tx))
    f = [str(x) for x in ref[f"{name}_files"]]
    return str(tmp_path / f[0]), str(tmp_path / f[1])


def _numbering(f, geom, cond):
    sizes = np.zeros(6, np.int64)
    assert f(geom.encode(), cond.encode(), sizes.ctypes.data, None, None, None, None, None, 0, 0, 0) == 0
    nmesh, nv, nvg, nt, N, nP = (int(x) for x in sizes)
    V = np.zeros((nv, 3))
    vglob, tidx = np.zeros(nv, np.int64), np.zeros(nt, np.int64)
    orient, barrier = np.zeros(nmesh, np.int32), np.zeros(nmesh, np.int32)
    assert f(geom.encode(), cond.encode(), sizes.ctypes.data, V.ctypes.data, vglob.ctypes.data, tidx.ctypes.data,
             orient.ctypes.data, barrier.ctypes.data, nv, nt, nmesh) == 0
    return dict(nmesh=nmesh, nv=nv, nvg=nvg, nt=nt, N=N, nP=nP, V=V, vglob=vglob, tidx=tidx, orient=orient,
                barrier=barrier)


@pytest.mark.parametrize("name", ["HeadMN1", "HeadMN2", "HeadMN3", "HeadNNb1"])
def test_numbering_matches_oracle(hook, ref, name, tmp_path):
    from oracle import oracle
    from openmeeg_gb300 import io
    geom, cond = _files(ref, name, tmp_path)
    h = _numbering(hook, geom, cond)
    g = oracle.digest(io.load_head(geom, cond))
    assert h["nv"] == h["nvg"] == g.V.shape[0]            # no shared vertices on these heads
    assert np.array_equal(h["vglob"], np.arange(h["nv"]))
    assert np.array_equal(h["V"], g.V)
    assert h["N"] == g.N
    assert np.array_equal(h["orient"], np.asarray(g.orient))
    assert np.array_equal(h["barrier"], np.asarray(g.barrier))
    assert np.array_equal(h["tidx"], np.asarray(g.tidx))
    assert h["N"] == ref[f"{name}_dsm"].shape[0]            # the reference's own DipSourceMat rows


@pytest.mark.parametrize("name", ["HeadNNa1", "HeadNNc1"])
def test_shared_vertex_copies(hook, ref, name, tmp_path):
    geom, cond = _files(ref, name, tmp_path)
    h = _numbering(hook, geom, cond)
    V, vg = h["V"], h["vglob"]
    assert h["nvg"] < h["nv"]
    # one id per distinct coordinate triple, shared exactly by the copies with equal coordinates
    _, inv = np.unique(V, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    assert len(np.unique(inv)) == h["nvg"] == len(np.unique(vg))
    pairs = np.unique(np.stack([inv, vg], 1), axis=0)
    assert len(pairs) == h["nvg"]
    # ids in order of first appearance
    _, first = np.unique(vg, return_index=True)
    assert np.all(np.diff(first) > 0) and vg[0] == 0
    # triangles after the vertices, the non-barrier ones filling the unknowns up to N
    assert h["N"] == ref[f"{name}_dsm"].shape[0]
    inner = h["tidx"] < h["N"]
    assert np.array_equal(np.sort(h["tidx"][inner]), np.arange(h["nvg"], h["N"]))
    assert h["N"] - h["nvg"] == h["nP"]
