"""Generates the golden fixtures of tests/golden/ by running the reference
OpenMEEG command-line tools (built from the reference sources by
oracle/ref/Makefile into oracle/_ref/).  Run where the reference sources are
available:

    python tests/golden/make_golden.py [--big]

Each fixture is an .npz of the reference's own outputs (read from its .bin
files) for a seeded workload of openmeeg_gb300.workloads:
  small_ico1_3l      HM (packed), DSM, H2EM, H2MM, DS2MM, EEG/MEG adjoint gains
  small_ico1_4l_out  same, 4 layers, outward-oriented meshes (interfaces flipped)
  small_ico2_3l_pert gains + DSM, SH-perturbed ico2 head
  config0            EEG/MEG adjoint gains of config0 (ico3, N=4486), 200 dipoles
  config1_200        (--big) EEG/MEG adjoint gains of config1 (ico4, N=17926) for
                     its first 200 dipoles
  head3_analytic     the reference's sample head Head3 (meshes, domains, dipoles,
                     128 electrodes, 162 magnetometers) with the analytic EEG and
                     MEG values its test suite compares against
                     (tests/analytic/eeg_head3_analytic.txt, meg_analytic.txt);
                     `--analytic-only` writes just this fixture
  reference_heads    the reference's sample heads HeadNNb1 (two extra spheres inside the
                     brain: non-nested), HeadNNa1 / HeadNNc1 (the brain cut into two
                     hemispheres whose interfaces share the cut mesh and its vertices) and
                     HeadMN1-3 (several non-conductive domains)
                     through om_assemble / om_gain with their own dipoles, patches and
                     squids, with the geometry files' texts; `--heads-only` writes just
                     this fixture (and head3_analytic)
  eit_sources        EITSourceMat (om_assemble -EITSM) for point electrodes and for
                     electrodes with radii on small_ico1_3l, small_ico1_4l_out and
                     small_ico2_3l_pert; `--eit-only` writes just this fixture (and
                     head3_analytic)
  internal_potentials Surf2VolMat and DipSource2InternalPotMat (om_assemble -H2IPM /
                     -DS2IPM, own domains and a forced one) at points in every layer
                     and in the air of small_ico1_3l and small_ico1_4l_out;
                     `--ipm-only` writes this fixture and the ones above
  direct_gains       om_minverser + om_gain -EEG / -MEG (the explicit-inverse pipeline of the
                     reference's own tests) on small_ico1_3l, small_ico2_3l_pert and config0,
                     with the reference's packed inverse of small_ico1_3l; `--direct-only`
                     writes just this fixture
  surface_sources    SurfSourceMat and SurfSource2MEGMat (om_assemble -SSM / -SS2MM)
                     of a source icosphere (ico1, r = 0.5, off-centre) in the brain of
                     small_ico1_3l and of small_ico1_4l_out; `--ssm-only` writes just
                     this fixture
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_runner  # noqa: E402
from openmeeg_gb300 import io, workloads  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def save(name, w, R, keep_hm=False):
    d = {"dipoles": w.dipoles, "electrodes": w.electrodes, "squids": w.squids}
    for k in ("dsm", "h2em", "h2mm", "ds2mm", "eeg", "meg"):
        if k in R:
            d[k] = R[k]
    if keep_hm:
        d["hm_packed"] = io.packed_upper(R["hm"])
    d["times"] = np.array([R["times"].get(k, np.nan) for k in ("hm", "dsm", "h2em", "h2mm", "ds2mm", "eeg", "meg")])
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **d)
    print(name, {k: (v.shape if hasattr(v, "shape") else v) for k, v in d.items()}, R["times"])


def save_head3_analytic():
    R = ref_runner.REFERENCE_DIR
    d3 = os.path.join(R, "data", "Head3")
    meshes, domains = io.read_geom(os.path.join(d3, "Head3.geom"))
    cond = io.read_cond(os.path.join(d3, "Head3.cond"))
    V, T = [], []
    for m in meshes:
        v, t = io.read_tri(m)
        V.append(v)
        T.append(t)
    names = [d[0] for d in domains]
    d = {"nverts": np.array([v.shape[0] for v in V]), "ntris": np.array([t.shape[0] for t in T]),
         "vertices": np.vstack(V), "triangles": np.vstack(T),
         "dom_nb": np.array([len(dm[1]) for dm in domains]),
         "dom_bounds": np.array([b for dm in domains for b in dm[1]]),
         "dom_sigma": np.array([cond[n] for n in names]), "dom_names": np.array(names),
         "dipoles": np.loadtxt(os.path.join(d3, "Head3.dip")),
         "electrodes": np.loadtxt(os.path.join(d3, "Head3.patches")),
         "squids": np.loadtxt(os.path.join(d3, "Head3.squids"), usecols=range(1, 8)),
         "eeg_analytic": np.loadtxt(os.path.join(R, "tests", "analytic", "eeg_head3_analytic.txt")),
         "meg_analytic": np.loadtxt(os.path.join(R, "tests", "analytic", "meg_analytic.txt"))}
    np.savez_compressed(os.path.join(OUT, "head3_analytic.npz"), **d)
    print("head3_analytic", {k: v.shape for k, v in d.items()})


def save_surface_sources():
    import subprocess
    import tempfile
    from openmeeg_gb300 import synthetic as syn
    if not ref_runner.available():
        ref_runner.build()
    V, T = syn.icosphere(1, inward=False)
    V = V * 0.5 + np.array([0.05, -0.03, 0.02])
    d = {"src_vertices": V, "src_triangles": T}
    for tag, w in (("3l", workloads.small(1, layers=3)), ("4l_out", workloads.small(1, layers=4, inward=False))):
        wd = tempfile.mkdtemp()
        ref_runner.write_head(wd, w.head, squids=w.squids)
        io.write_tri(os.path.join(wd, "src.tri"), V, T)
        for args in (["om_assemble", "-SSM", "head.geom", "head.cond", "src.tri", "ssm.bin"],
                     ["om_assemble", "-SS2MM", "src.tri", "meg.txt", "ss2mm.bin"]):
            subprocess.check_call([os.path.join(ref_runner.REF_BIN, args[0]), *args[1:]], cwd=wd,
                                  stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        d[f"ssm_{tag}"] = io.read_bin(os.path.join(wd, "ssm.bin"))[1]
        d[f"ss2mm_{tag}"] = io.read_bin(os.path.join(wd, "ss2mm.bin"))[1]
        d[f"squids_{tag}"] = w.squids
    np.savez_compressed(os.path.join(OUT, "surface_sources.npz"), **d)
    print("surface_sources", {k: v.shape for k, v in d.items()})


def internal_points(head, radii, seed, n_dirs=5):
    """Points along vertex directions of the innermost mesh (where every nested
    icosphere reaches its nominal radius, so a radius between two surfaces
    names the layer) at each radius, plus a few generic points deep in the
    innermost layer; shuffled so that dropped points sit between kept ones."""
    rng = np.random.default_rng(seed)
    V0 = head.vertices[0]
    dirs = V0[rng.choice(len(V0), n_dirs, replace=False)]
    dirs = dirs / np.linalg.norm(dirs, axis=1, keepdims=True)
    P = [d * r for d in dirs for r in radii]
    g = rng.standard_normal((4, 3))
    P += list(g / np.linalg.norm(g, axis=1, keepdims=True) * 0.4)
    P = np.array(P)
    return P[rng.permutation(len(P))]


def save_internal_potentials():
    """Surf2VolMat (om_assemble -H2IPM) and DipSource2InternalPotMat
    (-DS2IPM, with and without a forced domain) on two small heads."""
    import subprocess
    import tempfile
    if not ref_runner.available():
        ref_runner.build()
    d = {}
    cases = (("3l", workloads.small(1, layers=3), [0.3, 0.6, 0.895, 0.96, 1.1], "Scalp"),
             ("4l_out", workloads.small(1, layers=4, inward=False), [0.5, 0.865, 0.9, 0.96, 1.2], "CSF"))
    for k, (tag, w, radii, forced) in enumerate(cases):
        wd = tempfile.mkdtemp()
        ref_runner.write_head(wd, w.head, dipoles=w.dipoles)
        pts = internal_points(w.head, radii, workloads.SEED + 40 + k)
        io.write_matrix_txt(os.path.join(wd, "pts.txt"), pts)
        for args in (["om_assemble", "-H2IPM", "head.geom", "head.cond", "pts.txt", "h2ipm.bin"],
                     ["om_assemble", "-DS2IPM", "head.geom", "head.cond", "dip.txt", "pts.txt", "ds2ipm.bin"],
                     ["om_assemble", "-DS2IPM", "head.geom", "head.cond", "dip.txt", "pts.txt", "ds2ipm_f.bin",
                      forced]):
            subprocess.check_call([os.path.join(ref_runner.REF_BIN, args[0]), *args[1:]], cwd=wd,
                                  stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        d[f"points_{tag}"] = pts
        d[f"h2ipm_{tag}"] = io.read_bin(os.path.join(wd, "h2ipm.bin"))[1]
        d[f"ds2ipm_{tag}"] = io.read_bin(os.path.join(wd, "ds2ipm.bin"))[1]
        d[f"ds2ipm_forced_{tag}"] = io.read_bin(os.path.join(wd, "ds2ipm_f.bin"))[1]
        d[f"forced_{tag}"] = np.array(forced)
    np.savez_compressed(os.path.join(OUT, "internal_potentials.npz"), **d)
    print("internal_potentials", {k: v.shape for k, v in d.items()})


def save_eit():
    """EITSourceMat (om_assemble -EITSM) for point electrodes (3 columns) and
    for electrodes with radii (4 columns, some zero, some spanning several
    scalp triangles) on three small heads."""
    import subprocess
    import tempfile
    if not ref_runner.available():
        ref_runner.build()
    d = {}
    cases = (("3l", workloads.small(1, layers=3)), ("4l_out", workloads.small(1, layers=4, inward=False)),
             ("ico2_pert", workloads.small(2, layers=3, perturb=True)))
    for k, (tag, w) in enumerate(cases):
        rng = np.random.default_rng(workloads.SEED + 60 + k)
        el = w.electrodes[:, :3]
        rad = rng.choice([0.0, 0.05, 0.12, 0.2, 0.33], size=el.shape[0])
        wd = tempfile.mkdtemp()
        ref_runner.write_head(wd, w.head)
        io.write_matrix_txt(os.path.join(wd, "el3.txt"), el)
        io.write_matrix_txt(os.path.join(wd, "el4.txt"), np.hstack([el, rad[:, None]]))
        for args in (["om_assemble", "-EITSM", "head.geom", "head.cond", "el3.txt", "eit3.bin"],
                     ["om_assemble", "-EITSM", "head.geom", "head.cond", "el4.txt", "eit4.bin"]):
            subprocess.check_call([os.path.join(ref_runner.REF_BIN, args[0]), *args[1:]], cwd=wd,
                                  stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        d[f"electrodes_{tag}"] = np.hstack([el, rad[:, None]])
        d[f"eit_points_{tag}"] = io.read_bin(os.path.join(wd, "eit3.bin"))[1]
        d[f"eit_radii_{tag}"] = io.read_bin(os.path.join(wd, "eit4.bin"))[1]
    np.savez_compressed(os.path.join(OUT, "eit_sources.npz"), **d)
    print("eit_sources", {k: v.shape for k, v in d.items()})


def save_direct_gains():
    """The documented pipeline of the reference's own tests (TestHead.cmake): om_minverser
    (DSPTRF + DSPTRI) then om_gain -EEG / -MEG with the explicit inverse, on small_ico1_3l,
    small_ico2_3l_pert and config0."""
    import subprocess
    import tempfile
    if not ref_runner.available():
        ref_runner.build()
    d = {}
    cases = (("ico1_3l", workloads.small(1, layers=3)), ("ico2_3l_pert", workloads.small(2, layers=3, perturb=True)),
             ("config0", workloads.config0()))
    for tag, w in cases:
        wd = tempfile.mkdtemp()
        ref_runner.write_head(wd, w.head, w.dipoles, w.electrodes, w.squids)
        g, c = "head.geom", "head.cond"
        for args in (["om_assemble", "-HM", g, c, "hm.bin"], ["om_minverser", "hm.bin", "hminv.bin"],
                     ["om_assemble", "-DSM", g, c, "dip.txt", "dsm.bin"],
                     ["om_assemble", "-H2EM", g, c, "eeg.txt", "h2em.bin"],
                     ["om_assemble", "-H2MM", g, c, "meg.txt", "h2mm.bin"],
                     ["om_assemble", "-DS2MM", "dip.txt", "meg.txt", "ds2mm.bin"],
                     ["om_gain", "-EEG", "hminv.bin", "dsm.bin", "h2em.bin", "geeg.bin"],
                     ["om_gain", "-MEG", "hminv.bin", "dsm.bin", "h2mm.bin", "ds2mm.bin", "gmeg.bin"]):
            subprocess.check_call([os.path.join(ref_runner.REF_BIN, args[0]), *args[1:]], cwd=wd,
                                  stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        d[f"eeg_{tag}"] = io.read_bin(os.path.join(wd, "geeg.bin"))[1]
        d[f"meg_{tag}"] = io.read_bin(os.path.join(wd, "gmeg.bin"))[1]
        if tag == "ico1_3l":   # the reference's explicit inverse of the smallest head (N = 286)
            d[f"hminv_packed_{tag}"] = io.packed_upper(io.read_bin(os.path.join(wd, "hminv.bin"))[1])
        import shutil
        shutil.rmtree(wd, ignore_errors=True)
    np.savez_compressed(os.path.join(OUT, "direct_gains.npz"), **d)
    print("direct_gains", {k: v.shape for k, v in d.items()})


HEAD1_INPUTS = ("Head1.geom", "Head1.cond", "cortex.1.tri", "skull.1.tri", "scalp.1.tri", "Head1.dip",
                "Head1.patches", "Head1.squids", "Head1.tri")
HEAD1_MATS = ("Head1.hm", "Head1.hm_inv", "Head1.dsm", "Head1.h2em", "Head1.h2mm", "Head1.ds2mm", "Head1.dgem",
              "Head1.dgmm", "Head1.ssm", "Head1.sgem")


def save_head1():
    """The reference's own golden files for its Head1 test head
    (tests/initialTest/Head1.*: MATLAB v7.3 / HDF5, written by its MatlabIO) and
    the inputs they were made from (data/Head1), copied into tests/golden/head1/
    so the tests can read them (openmeeg_gb300.matio) without the reference."""
    import shutil
    R = ref_runner.REFERENCE_DIR
    dst = os.path.join(OUT, "head1")
    os.makedirs(dst, exist_ok=True)
    for f in HEAD1_INPUTS:
        shutil.copyfile(os.path.join(R, "data", "Head1", f), os.path.join(dst, f))
    for f in HEAD1_MATS:
        shutil.copyfile(os.path.join(R, "tests", "initialTest", f), os.path.join(dst, f))
    print("head1", sorted(os.listdir(dst)))


def cortical_probe(head) -> np.ndarray:
    """The seeded random vector the config0 cortical fixtures are projected on."""
    n = sum(v.shape[0] for v in head.vertices) + sum(t.shape[0] for t in head.triangles[:-1])
    return np.random.default_rng(2024).standard_normal(n)


def save_cortical():
    """om_assemble -CM (CorticalMat with automatic and given alpha / beta,
    CorticalMat2 with gamma) on the reference's Head1 with its EEG patches and
    its test's "Brain" domain and parameters (TestHead.cmake:94-96), and on the
    seeded small_ico1_3l head.  Head1's mesh / .geom / .cond texts and patches
    are stored so a test can rebuild the files without the reference.  Head1's
    CorticalMat2 is not kept: two of its 32 patches give linearly dependent rows
    of Head2EEGMat (rank 31), so H G^-1 H^T is singular and the reference's
    inverse of it returns rounding noise."""
    import subprocess
    import tempfile
    R = ref_runner.REFERENCE_DIR
    if not ref_runner.available():
        ref_runner.build()
    d = {}
    variants = (("auto", []), ("ab", ["1e-4", "1.58e-2"]), ("gamma", ["12.4"]))

    def run(wd, geom, cond, eeg, tag, args):
        subprocess.check_call([os.path.join(ref_runner.REF_BIN, "om_assemble"), "-CM", geom, cond, eeg, "Brain",
                               "cm.bin", *args], cwd=wd, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        return io.read_bin(os.path.join(wd, "cm.bin"))[1]

    base = os.path.join(R, "data", "Head1")
    files = ["Head1.geom", "Head1.cond", "cortex.1.tri", "skull.1.tri", "scalp.1.tri", "Head1.patches"]
    d["head1_files"] = np.array(files)
    d["head1_texts"] = np.array([open(os.path.join(base, f)).read() for f in files])
    for tag, args in variants[:2]:
        d[f"head1_{tag}"] = run(base, "Head1.geom", "Head1.cond", "Head1.patches", tag, args)
    w = workloads.small(1, layers=3)
    wd = tempfile.mkdtemp()
    ref_runner.write_head(wd, w.head, w.dipoles, w.electrodes, w.squids)
    for tag, args in variants:
        d[f"ico1_3l_{tag}"] = run(wd, "head.geom", "head.cond", "eeg.txt", tag, args)
    import shutil
    shutil.rmtree(wd, ignore_errors=True)
    # config0 (N = 4486, 64 electrodes): too large to store whole; kept as the column 2-norms and the
    # projection X^T u on a seeded random vector u (cortical_probe)
    w = workloads.config0()
    wd = tempfile.mkdtemp()
    ref_runner.write_head(wd, w.head, w.dipoles, w.electrodes, w.squids)
    u = cortical_probe(w.head)
    for tag, args in variants:
        X = run(wd, "head.geom", "head.cond", "eeg.txt", tag, args)
        d[f"config0_{tag}_norms"] = np.linalg.norm(X, axis=0)
        d[f"config0_{tag}_proj"] = X.T @ u
    shutil.rmtree(wd, ignore_errors=True)
    np.savez_compressed(os.path.join(OUT, "cortical.npz"), **d)
    print("cortical", {k: v.shape for k, v in d.items()})


def save_shared_vertex_sources():
    """om_assemble -SSM, -H2IPM and -EITSM on the reference's HeadNNa1, whose
    two hemispheres share the vertices of their cut mesh: an ico1 source
    surface in the north hemisphere, points inside both hemispheres (plus two
    in the air, dropped) and the head's own EEG patches as point electrodes.
    The head's files are in reference_heads.npz."""
    import subprocess
    import shutil
    import tempfile
    from openmeeg_gb300 import synthetic as syn
    R = ref_runner.REFERENCE_DIR
    if not ref_runner.available():
        ref_runner.build()
    wd = tempfile.mkdtemp()
    base = os.path.join(R, "data", "HeadNNa1")
    for f in os.listdir(base):
        shutil.copy(os.path.join(base, f), wd)
    V, T = syn.icosphere(1, inward=False)
    V = V * 0.08 + np.array([0.02, -0.01, 0.45])
    rng = np.random.default_rng(5)
    P = []
    while len(P) < 16:   # inside the hemispheres, away from the cut and the cortex
        x = rng.uniform(-0.7, 0.7, 3)
        if np.linalg.norm(x) < 0.7 and abs(x[2]) > 0.1:
            P.append(x)
    P = np.array(P + [[1.3, 0.0, 0.0], [0.0, -1.3, 0.2]])
    io.write_tri(os.path.join(wd, "src.tri"), V, T)
    io.write_matrix_txt(os.path.join(wd, "pts.txt"), P)
    for args in (["om_assemble", "-SSM", "HeadNNa1.geom", "HeadNNa1.cond", "src.tri", "ssm.bin"],
                 ["om_assemble", "-H2IPM", "HeadNNa1.geom", "HeadNNa1.cond", "pts.txt", "h2ipm.bin"],
                 ["om_assemble", "-EITSM", "HeadNNa1.geom", "HeadNNa1.cond", "HeadNNa1.patches", "eit.bin"]):
        subprocess.check_call([os.path.join(ref_runner.REF_BIN, args[0]), *args[1:]], cwd=wd,
                              stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    d = {"src_vertices": V, "src_triangles": T, "points": P,
         "ssm": io.read_bin(os.path.join(wd, "ssm.bin"))[1], "h2ipm": io.read_bin(os.path.join(wd, "h2ipm.bin"))[1],
         "eit": io.read_bin(os.path.join(wd, "eit.bin"))[1],
         "eit_electrodes": io.read_sensors_txt(os.path.join(wd, "HeadNNa1.patches"))[1]}
    shutil.rmtree(wd, ignore_errors=True)
    np.savez_compressed(os.path.join(OUT, "shared_vertex_sources.npz"), **d)
    print("shared_vertex_sources", {k: v.shape for k, v in d.items()})


REFERENCE_HEADS = ("HeadNNb1", "HeadMN1", "HeadMN2", "HeadMN3", "HeadNNa1", "HeadNNc1")


def save_reference_heads():
    """The reference's non-nested (two extra spheres in the brain) and
    multiple-non-conductive sample heads, run through its own pipeline with its
    own dipoles, EEG patches and MEG squids.  The .geom / .cond / mesh texts are
    stored so that a test can rebuild the files without the reference."""
    R = ref_runner.REFERENCE_DIR
    if not ref_runner.available():
        ref_runner.build()
    d = {}
    for name in REFERENCE_HEADS:
        base = os.path.join(R, "data", name)
        geom, cond = os.path.join(base, name + ".geom"), os.path.join(base, name + ".cond")
        dip, eeg, meg = (os.path.join(base, name + ext) for ext in (".dip", ".patches", ".squids"))
        out = ref_runner.run_pipeline_files(geom, cond, dip, eeg, meg)
        meshes, _, _ = io.read_geom_full(geom)
        d[f"{name}_files"] = np.array([os.path.basename(geom), os.path.basename(cond)] +
                                      [os.path.basename(p) for _, p in meshes])
        d[f"{name}_texts"] = np.array([open(geom).read(), open(cond).read()] + [open(p).read() for _, p in meshes])
        d[f"{name}_dipoles"] = io.read_matrix_txt(dip)
        d[f"{name}_electrodes"] = io.read_sensors_txt(eeg)[1]
        d[f"{name}_squids"] = io.read_sensors_txt(meg)[1]
        if name in ("HeadNNb1", "HeadMN3", "HeadNNa1"):   # head matrices and H2MM of three (fixture size)
            d[f"{name}_hm_packed"] = io.packed_upper(out["hm"])
        for k in ("dsm", "h2em", "h2mm", "ds2mm", "eeg", "meg"):
            if k != "h2mm" or name in ("HeadNNb1", "HeadMN3", "HeadNNa1"):
                d[f"{name}_{k}"] = out[k]
        ana = os.path.join(R, "tests", "analytic", f"eeg_head{name[4:]}_analytic.txt")
        if os.path.exists(ana):   # the analytic EEG values the reference's tests compare against
            d[f"{name}_eeg_analytic"] = np.loadtxt(ana)
        print(name, {k: out[k].shape for k in out})
    np.savez_compressed(os.path.join(OUT, "reference_heads.npz"), **d)


def main():
    if "--direct-only" in sys.argv:
        save_direct_gains()
        return
    if "--cortical-only" in sys.argv:
        save_cortical()
        return
    if "--head1-only" in sys.argv:
        save_head1()
        return
    if "--shared-only" in sys.argv:
        save_shared_vertex_sources()
        return
    save_head3_analytic()
    if "--analytic-only" in sys.argv:
        return
    save_reference_heads()
    if "--heads-only" in sys.argv:
        return
    save_eit()
    if "--eit-only" in sys.argv:
        return
    save_internal_potentials()
    if "--ipm-only" in sys.argv:
        return
    save_surface_sources()
    if "--ssm-only" in sys.argv:
        return
    save_direct_gains()
    save_cortical()
    save_head1()
    save_shared_vertex_sources()
    if not ref_runner.available():
        ref_runner.build()
    big = "--big" in sys.argv
    w = workloads.small(1, layers=3)
    save("small_ico1_3l", w, ref_runner.run_pipeline(w.head, w.dipoles, w.electrodes, w.squids), keep_hm=True)
    w = workloads.small(1, layers=4, inward=False)
    save("small_ico1_4l_out", w, ref_runner.run_pipeline(w.head, w.dipoles, w.electrodes, w.squids), keep_hm=True)
    w = workloads.small(2, layers=3, perturb=True)
    R = ref_runner.run_pipeline(w.head, w.dipoles, w.electrodes, w.squids)
    R.pop("hm")
    R.pop("h2mm")
    save("small_ico2_3l_pert", w, R)
    w = workloads.config0()
    R = ref_runner.run_pipeline(w.head, w.dipoles, w.electrodes, w.squids, want=("hm", "h2em", "h2mm", "ds2mm",
                                                                                  "eeg", "meg"))
    for k in ("hm", "h2mm", "h2em"):
        R.pop(k)
    save("config0", w, R)
    if big:
        w = workloads.config1(200)
        t0 = time.time()
        R = ref_runner.run_pipeline(w.head, w.dipoles, w.electrodes, w.squids,
                                    want=("hm", "h2em", "h2mm", "ds2mm", "eeg", "meg"))
        for k in ("hm", "h2mm", "h2em", "ds2mm"):
            R.pop(k)
        save("config1_200", w, R)
        print("config1 reference run", time.time() - t0, "s")


if __name__ == "__main__":
    main()
