"""CPU tests: the oracle restatement against the reference's own outputs
(golden fixtures), file formats, and the C ABI library's exported symbols."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden, rel


def _w(name):
    from openmeeg_gb300 import workloads
    return {
        "small_ico1_3l": lambda: workloads.small(1, layers=3),
        "small_ico1_4l_out": lambda: workloads.small(1, layers=4, inward=False),
        "small_ico2_3l_pert": lambda: workloads.small(2, layers=3, perturb=True),
    }[name]()


@pytest.mark.parametrize("name", ["small_ico1_3l", "small_ico1_4l_out"])
def test_oracle_headmat_pinned_to_reference(name):
    from oracle import oracle
    from openmeeg_gb300 import io
    G = golden(name)
    w = _w(name)
    g = oracle.digest(w.head)
    HM = oracle.headmat(g)
    ref = io.unpack_upper(G["hm_packed"], g.N)
    assert rel(HM, ref) < 1e-14


@pytest.mark.parametrize("name", ["small_ico1_3l", "small_ico1_4l_out", "small_ico2_3l_pert", "config0"])
def test_oracle_forward_pipeline_pinned_to_reference(name):
    """The reference pipeline the CPU baseline times (packed head matrix,
    DSPTRF/DSPTRS solve of the stacked sensor rows, DipSourceMat, contraction)
    gives the reference's own gains."""
    from oracle import oracle
    from openmeeg_gb300 import workloads
    G = golden(name)
    w = workloads.config0() if name == "config0" else _w(name)
    ge, gm, t = oracle.forward_pipeline(w.head, w.dipoles, w.electrodes, w.squids)
    assert rel(ge, G["eeg"]) < 1e-12
    assert rel(gm, G["meg"]) < 1e-12
    assert {"headmat", "factor_solve", "dsm", "contract"} <= set(t)


def test_oracle_direct_gains_pinned_to_reference():
    """om_minverser + om_gain -EEG / -MEG: the oracle's DSPTRF + DSPTRI inverse
    of the reference's head matrix equals the reference's own inverse, and the
    direct-form gains from it equal the reference's direct-form gains."""
    from oracle import oracle
    from openmeeg_gb300 import io
    D = golden("direct_gains")
    G = golden("small_ico1_3l")
    w = _w("small_ico1_3l")
    g = oracle.digest(w.head)
    inv = oracle.invert_packed(G["hm_packed"], g.N)
    assert rel(inv, D["hminv_packed_ico1_3l"]) < 1e-13
    HMinv = io.unpack_upper(inv, g.N)
    assert rel(oracle.gain_eeg_direct(HMinv, G["dsm"], G["h2em"]), D["eeg_ico1_3l"]) < 1e-13
    assert rel(oracle.gain_meg_direct(HMinv, G["dsm"], G["h2mm"], G["ds2mm"]), D["meg_ico1_3l"]) < 1e-13
    # the explicit-inverse and the adjoint pipelines agree
    assert rel(D["eeg_ico1_3l"], G["eeg"]) < 1e-12 and rel(D["meg_ico1_3l"], G["meg"]) < 1e-12


def test_packed_bunch_kaufman_solve():
    """DSPTRF/DSPTRS on packed-upper storage (SymMatrix::solveLin) on an
    indefinite symmetric matrix, against a dense solve."""
    from oracle import oracle
    from openmeeg_gb300 import io
    rng = np.random.default_rng(1)
    n = 200
    A = rng.standard_normal((n, n))
    A = A + A.T + np.diag(np.where(np.arange(n) % 2 == 0, 20.0, -20.0))
    B = rng.standard_normal((n, 5))
    X = oracle.solve_lin_packed(io.packed_upper(A), n, B)
    assert rel(X, np.linalg.solve(A, B)) < 1e-12
    with pytest.raises(ValueError):
        oracle.solve_lin_packed(io.packed_upper(A)[:-1], n, B)


@pytest.mark.parametrize("name", ["small_ico1_3l", "small_ico1_4l_out", "small_ico2_3l_pert"])
def test_oracle_sources_sensors_gains_pinned_to_reference(name):
    from oracle import oracle
    G = golden(name)
    w = _w(name)
    g = oracle.digest(w.head)
    D = oracle.dsm(g, w.dipoles)
    assert rel(D, G["dsm"]) < 1e-14
    E = oracle.h2em(g, w.electrodes)
    assert rel(E, G["h2em"]) < 1e-14
    M = oracle.h2mm(g, w.squids)
    if "h2mm" in G:
        assert rel(M, G["h2mm"]) < 1e-11
    S = oracle.ds2mm(w.dipoles, w.squids)
    assert rel(S, G["ds2mm"]) < 1e-14
    HM = oracle.headmat(g)
    assert rel(oracle.gain_eeg(HM, D, E), G["eeg"]) < 1e-12
    assert rel(oracle.gain_meg(HM, D, M, S), G["meg"]) < 1e-12


@pytest.mark.parametrize("tag,layers,inward", [("3l", 3, True), ("4l_out", 4, False)])
def test_oracle_internal_potentials_pinned_to_reference(tag, layers, inward):
    """Surf2VolMat and DipSource2InternalPotMat (own domains and a forced one)
    against om_assemble -H2IPM / -DS2IPM; points in the air are dropped."""
    from oracle import oracle
    from openmeeg_gb300 import workloads
    G = golden("internal_potentials")
    w = workloads.small(1, layers=layers, inward=inward)
    g = oracle.digest(w.head)
    pts = G[f"points_{tag}"]
    H = oracle.surf2volmat(g, pts)
    assert H.shape == G[f"h2ipm_{tag}"].shape and H.shape[0] < pts.shape[0]
    assert rel(H, G[f"h2ipm_{tag}"]) < 1e-14
    assert rel(oracle.dipsource2internalpotmat(g, w.dipoles, pts), G[f"ds2ipm_{tag}"]) < 1e-14
    forced = str(G[f"forced_{tag}"])
    assert rel(oracle.dipsource2internalpotmat(g, w.dipoles, pts, forced), G[f"ds2ipm_forced_{tag}"]) < 1e-14


@pytest.mark.parametrize("tag,kw", [("3l", dict(layers=3)), ("4l_out", dict(layers=4, inward=False)),
                                    ("ico2_pert", dict(subdiv=2, layers=3, perturb=True))])
def test_oracle_eit_source_pinned_to_reference(tag, kw):
    """EITSourceMat against om_assemble -EITSM, point electrodes and electrodes
    with radii (flood-filled injection triangles)."""
    from oracle import oracle
    from openmeeg_gb300 import workloads
    G = golden("eit_sources")
    w = workloads.small(**{"subdiv": 1, **kw})
    g = oracle.digest(w.head)
    el = G[f"electrodes_{tag}"]
    assert rel(oracle.eitsourcemat(g, el[:, :3]), G[f"eit_points_{tag}"]) < 1e-14
    assert rel(oracle.eitsourcemat(g, el), G[f"eit_radii_{tag}"]) < 1e-14


@pytest.mark.parametrize("name", ["HeadNNb1", "HeadMN1", "HeadMN2", "HeadMN3"])
def test_oracle_reference_heads_pinned_to_reference(name, tmp_path):
    """The reference's non-nested and multiple-non-conductive sample heads, read
    from its own files through io.load_head: matrices at rounding level; gains
    at 1e-10, except on the two heads whose head matrix is singular (see
    tests/test_gpu_reference_heads.py), where the null direction the sensors do
    not see leaves the solvers 3e-6 apart -- checked at 1e-4 and against the
    reference's analytic EEG values with its tolerances."""
    import warnings
    from oracle import analytic, oracle
    from openmeeg_gb300 import io
    G = golden("reference_heads")
    for fn, tx in zip(G[f"{name}_files"], G[f"{name}_texts"]):
        (tmp_path / str(fn)).write_text(str(tx))
    f = [str(x) for x in G[f"{name}_files"]]
    head = io.load_head(str(tmp_path / f[0]), str(tmp_path / f[1]))
    g = oracle.digest(head)
    HM = oracle.headmat(g)
    if f"{name}_hm_packed" in G:
        assert rel(HM, io.unpack_upper(G[f"{name}_hm_packed"], g.N)) < 1e-14
    D = oracle.dsm(g, G[f"{name}_dipoles"])
    E = oracle.h2em(g, G[f"{name}_electrodes"])
    M = oracle.h2mm(g, G[f"{name}_squids"])
    S = oracle.ds2mm(G[f"{name}_dipoles"], G[f"{name}_squids"])
    assert rel(D, G[f"{name}_dsm"]) < 1e-14
    assert rel(E, G[f"{name}_h2em"]) < 1e-14
    if f"{name}_h2mm" in G:
        assert rel(M, G[f"{name}_h2mm"]) < 1e-11
    assert rel(S, G[f"{name}_ds2mm"]) < 1e-14
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")   # LAPACK's ill-conditioning warning on the singular heads
        ge, gm = oracle.gain_eeg(HM, D, E), oracle.gain_meg(HM, D, M, S)
    tol = 1e-4 if name in ("HeadMN1", "HeadMN2") else 1e-10
    assert rel(ge, G[f"{name}_eeg"]) < tol and rel(gm, G[f"{name}_meg"]) < tol
    if f"{name}_eeg_analytic" in G:
        ana = G[f"{name}_eeg_analytic"]
        assert np.all(analytic.rdm(ge, ana) < 0.10) and np.all(analytic.mag(ge, ana) < 0.10)


def test_text_formats(tmp_path):
    """Named .geom v1.1 (Meshes / Interfaces of +-mesh names / Domains of
    +-interface names), OFF meshes, sensor labels and plain dipole rows."""
    from openmeeg_gb300 import io
    from openmeeg_gb300 import synthetic as syn
    V, T = syn.icosphere(1, inward=False)
    with open(tmp_path / "a.off", "w") as f:
        f.write(f"OFF\n{V.shape[0]} {T.shape[0]} 0\n")
        f.writelines(f"{x} {y} {z}\n" for x, y, z in V * 0.5)
        f.writelines(f"3 {a} {b} {c}\n" for a, b, c in T)
    io.write_tri(str(tmp_path / "b.tri"), V, T)
    (tmp_path / "h.geom").write_text(
        "# Domain Description 1.1\nMeshes 2\nMesh inner: \"a.off\"\nMesh outer: \"b.tri\"\n"
        "Interfaces 2\nInterface In: +inner\nInterface Out: outer\n"
        "Domains 3\nDomain BRAIN: -In\nDomain SKIN: +In -Out\nDomain AIR: Out shared\n")
    (tmp_path / "h.cond").write_text("BRAIN 1\nSKIN 0.5\nAIR 0\n")
    head = io.load_head(str(tmp_path / "h.geom"), str(tmp_path / "h.cond"))
    assert head.names == ["inner", "outer"] and np.allclose(head.vertices[0], V * 0.5)
    assert head.domains == [("BRAIN", [-1], 1.0), ("SKIN", [1, -2], 0.5), ("AIR", [2], 0.0)]
    (tmp_path / "s.txt").write_text("E1 0.1 0.2 0.3\nE2 1 2.5 3\n")
    labels, vals = io.read_sensors_txt(str(tmp_path / "s.txt"))
    assert labels == ["E1", "E2"] and vals.shape == (2, 3)
    (tmp_path / "d.txt").write_text("0 0 0.4250  0.7 0 0.7\n")
    assert io.read_matrix_txt(str(tmp_path / "d.txt")).shape == (1, 6)


def test_oracle_numbering_and_pairs():
    """Unknown count and mesh pairs of nested heads (geometry.cpp:256-295, 405-420)."""
    from oracle import oracle
    from openmeeg_gb300 import synthetic as syn
    h3 = syn.nested_head(3, [0.87, 0.92, 1.0], [1.0, 0.0125, 1.0])
    g = oracle.digest(h3)
    assert g.N == 3 * 642 + 2 * 1280 == 4486
    assert g.pairs.tolist() == [[0, 0], [1, 0], [1, 1], [2, 1], [2, 2]]
    assert list(g.barrier) == [0, 0, 1]
    h4 = syn.nested_head(1, [0.85, 0.88, 0.92, 1.0], [0.33, 1.79, 0.0042, 0.33], inward=False)
    g4 = oracle.digest(h4)
    assert g4.N == 4 * 42 + 3 * 80
    assert list(g4.orient) == [-1, -1, -1, -1]


def test_bin_roundtrip(tmp_path):
    from openmeeg_gb300 import io
    rng = np.random.default_rng(1)
    A = rng.standard_normal((7, 5))
    io.write_bin(str(tmp_path / "a.bin"), A)
    k, B = io.read_bin(str(tmp_path / "a.bin"))
    assert k == "full" and np.array_equal(A, B)
    S = rng.standard_normal((6, 6))
    S = S + S.T
    io.write_bin(str(tmp_path / "s.bin"), S, kind="sym")
    raw = open(tmp_path / "s.bin", "rb").read()
    assert len(raw) == 4 + 8 * 21   # uint32 n + packed upper
    k, B = io.read_bin(str(tmp_path / "s.bin"))
    assert k == "sym" and np.array_equal(S, B)
    # packed-upper order is i + j(j+1)/2 (symmatrix.h:52-62)
    p = io.packed_upper(S)
    assert p[1 + 2 * 3 // 2] == S[1, 2]
    io.write_bin(str(tmp_path / "v.bin"), np.arange(4.0), kind="vector")
    assert io.read_bin(str(tmp_path / "v.bin"))[0] == "vector"
    io.write_bin(str(tmp_path / "sp.bin"), ([0, 2], [1, 3], [1.5, -2.0], 3, 4), kind="sparse")
    k, M = io.read_bin(str(tmp_path / "sp.bin"))
    assert k == "sparse" and M[0, 1] == 1.5 and M[2, 3] == -2.0


def test_geom_files_roundtrip(tmp_path):
    from openmeeg_gb300 import io, workloads
    from oracle import ref_runner
    w = workloads.small(1)
    ref_runner.write_head(str(tmp_path), w.head)
    meshes, doms = io.read_geom(str(tmp_path / "head.geom"))
    assert [os.path.basename(m) for m in meshes] == ["cortex.tri", "skull.tri", "scalp.tri"]
    assert doms == [(d[0], d[1]) for d in w.head.domains]
    V, T = io.read_tri(meshes[0])
    assert np.array_equal(V, w.head.vertices[0]) and np.array_equal(T, w.head.triangles[0])
    cond = io.read_cond(str(tmp_path / "head.cond"))
    assert cond["Skull"] == 0.0125


def _header_symbols():
    txt = open(os.path.join(ROOT, "include", "openmeeg_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(omg_\w+)\(", txt, re.M)))


def test_library_exports_every_declared_symbol():
    from openmeeg_gb300 import build, _lib
    path = build.build()
    lib = ctypes.CDLL(path)
    syms = _header_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(syms) <= set(_lib.EXPORTED) | set(syms)


def test_library_fails_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from openmeeg_gb300 import _lib
    lib = _lib.load()
    h = ctypes.c_void_p()
    rc = lib.omg_context_create(0, ctypes.byref(h))
    assert rc != 0
    assert lib.omg_last_error()


def test_analytic_sphere_series_pinned_to_reference_values():
    """The nested-sphere EEG series and Sarvas's MEG formula reproduce the
    analytic values the reference's test suite ships for its sample head
    Head3 (radii .87/.92/1, conductivities 1/.0125/1, 6 dipoles, 128
    electrodes, 162 magnetometers).  The MEG file holds 8 significant digits;
    dipole 6 is radial (zero field) and is checked in absolute terms."""
    from oracle import analytic as an
    d = golden("head3_analytic")
    V = an.eeg_sphere([0.87, 0.92, 1.0], [1.0, 0.0125, 1.0], d["dipoles"], d["electrodes"])
    assert an.rdm(V, d["eeg_analytic"]).max() < 1e-12
    assert an.mag(V, d["eeg_analytic"]).max() < 1e-12
    B = an.sarvas(d["dipoles"], d["squids"][:, :6])
    assert an.rdm(B[:, :5], d["meg_analytic"][:, :5]).max() < 1e-6
    assert an.mag(B[:, :5], d["meg_analytic"][:, :5]).max() < 1e-6
    assert np.abs(B[:, 5]).max() < 1e-12 * np.abs(B[:, :5]).max()


def test_analytic_series_single_layer_limit():
    """Three layers of equal conductivity are one homogeneous sphere: the
    series then equals the closed form of a dipole in a sphere, checked here
    against a four-layer split of the same sphere."""
    from oracle import analytic as an
    rng = np.random.default_rng(5)
    dip = np.hstack([rng.uniform(-0.4, 0.4, (4, 3)), rng.standard_normal((4, 3))])
    el = rng.standard_normal((20, 3))
    el /= np.linalg.norm(el, axis=1, keepdims=True)
    V3 = an.eeg_sphere([0.8, 0.9, 1.0], [0.7, 0.7, 0.7], dip, el)
    V4 = an.eeg_sphere([0.6, 0.85, 0.95, 1.0], [0.7, 0.7, 0.7, 0.7], dip, el)
    V1 = an.eeg_sphere([1.0], [0.7], dip, el)
    assert np.abs(V3 - V1).max() < 1e-12 * np.abs(V1).max()
    assert np.abs(V4 - V1).max() < 1e-12 * np.abs(V1).max()
