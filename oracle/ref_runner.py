"""Runs the reference OpenMEEG command-line tools (built by oracle/ref/Makefile
into oracle/_ref/) on a head model -- TEST INFRASTRUCTURE ONLY.

Used to pin the oracle restatement and to generate golden fixtures.  Only
works where the reference sources were available at build time.
"""
from __future__ import annotations

import os
import subprocess
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BIN = os.path.join(HERE, "_ref", "bin")
# Where the reference sources are read from (this recipe builds them where they
# lie); OMG_REFERENCE_DIR overrides it.
REFERENCE_DIR = os.environ.get("OMG_REFERENCE_DIR", "/root/reference")


def available() -> bool:
    return os.path.exists(os.path.join(REF_BIN, "om_assemble"))


def build(ref_src: str = REFERENCE_DIR, jobs: int = 8) -> bool:
    if not os.path.isdir(ref_src):
        return False
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"), f"REF={ref_src}", f"-j{jobs}"],
                          stdout=subprocess.DEVNULL)
    return available()


def write_head(d: str, head, dipoles=None, electrodes=None, squids=None):
    from openmeeg_gb300 import io
    files = []
    for k, (V, T) in enumerate(zip(head.vertices, head.triangles)):
        fn = f"{head.names[k]}.tri"
        io.write_tri(os.path.join(d, fn), V, T)
        files.append(fn)
    io.write_geom(os.path.join(d, "head.geom"), files, head.domains)
    io.write_cond(os.path.join(d, "head.cond"), head.domains)
    if dipoles is not None:
        io.write_matrix_txt(os.path.join(d, "dip.txt"), dipoles)
    if electrodes is not None:
        io.write_matrix_txt(os.path.join(d, "eeg.txt"), electrodes[:, :3])
    if squids is not None:
        io.write_matrix_txt(os.path.join(d, "meg.txt"), squids)


def _run(d, *args, threads=None):
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    t0 = time.perf_counter()
    subprocess.check_call([os.path.join(REF_BIN, args[0]), *args[1:]], cwd=d, env=env,
                          stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return time.perf_counter() - t0


def run_pipeline(head, dipoles, electrodes=None, squids=None, workdir=None, dsm_adaptive=True, threads=None,
                 want=("hm", "dsm", "h2em", "h2mm", "ds2mm", "eeg", "meg")):
    """Runs om_assemble (-HM -DSM -H2EM -H2MM -DS2MM) and om_gain -*adjoint.
    Returns a dict of numpy arrays plus per-stage wall times under 'times'."""
    from openmeeg_gb300 import io
    own = workdir is None
    d = workdir or tempfile.mkdtemp(prefix="omref_")
    write_head(d, head, dipoles, electrodes, squids)
    out, times = {}, {}
    geom, cond = "head.geom", "head.cond"
    if "hm" in want or "eeg" in want or "meg" in want:
        times["hm"] = _run(d, "om_assemble", "-HM", geom, cond, "hm.bin", threads=threads)
        out["hm"] = io.read_bin(os.path.join(d, "hm.bin"))[1]
    if "dsm" in want:
        times["dsm"] = _run(d, "om_assemble", "-DSM" if dsm_adaptive else "-DSMNA", geom, cond, "dip.txt",
                            "dsm.bin", threads=threads)
        out["dsm"] = io.read_bin(os.path.join(d, "dsm.bin"))[1]
    if electrodes is not None and ("h2em" in want or "eeg" in want):
        times["h2em"] = _run(d, "om_assemble", "-H2EM", geom, cond, "eeg.txt", "h2em.bin", threads=threads)
        out["h2em"] = io.read_bin(os.path.join(d, "h2em.bin"))[1]
    if squids is not None and ("h2mm" in want or "meg" in want):
        times["h2mm"] = _run(d, "om_assemble", "-H2MM", geom, cond, "meg.txt", "h2mm.bin", threads=threads)
        out["h2mm"] = io.read_bin(os.path.join(d, "h2mm.bin"))[1]
        times["ds2mm"] = _run(d, "om_assemble", "-DS2MM", "dip.txt", "meg.txt", "ds2mm.bin", threads=threads)
        out["ds2mm"] = io.read_bin(os.path.join(d, "ds2mm.bin"))[1]
    if electrodes is not None and "eeg" in want:
        times["eeg"] = _run(d, "om_gain", "-EEGadjoint", geom, cond, "dip.txt", "hm.bin", "h2em.bin", "geeg.bin",
                            threads=threads)
        out["eeg"] = io.read_bin(os.path.join(d, "geeg.bin"))[1]
    if squids is not None and "meg" in want:
        times["meg"] = _run(d, "om_gain", "-MEGadjoint", geom, cond, "dip.txt", "hm.bin", "h2mm.bin", "ds2mm.bin",
                            "gmeg.bin", threads=threads)
        out["meg"] = io.read_bin(os.path.join(d, "gmeg.bin"))[1]
    out["times"] = times
    if own:
        import shutil
        shutil.rmtree(d, ignore_errors=True)
    return out


def run_pipeline_files(geom, cond, dip, eeg=None, meg=None, threads=None,
                       want=("hm", "dsm", "h2em", "h2mm", "ds2mm", "eeg", "meg")):
    """Same stages as run_pipeline on existing input files (absolute paths)."""
    from openmeeg_gb300 import io
    d = tempfile.mkdtemp(prefix="omref_")
    out = {}
    stages = [("hm", ["om_assemble", "-HM", geom, cond, "hm.bin"]),
              ("dsm", ["om_assemble", "-DSM", geom, cond, dip, "dsm.bin"])]
    if eeg:
        stages.append(("h2em", ["om_assemble", "-H2EM", geom, cond, eeg, "h2em.bin"]))
    if meg:
        stages += [("h2mm", ["om_assemble", "-H2MM", geom, cond, meg, "h2mm.bin"]),
                   ("ds2mm", ["om_assemble", "-DS2MM", dip, meg, "ds2mm.bin"])]
    if eeg:
        stages.append(("eeg", ["om_gain", "-EEGadjoint", geom, cond, dip, "hm.bin", "h2em.bin", "eeg.bin"]))
    if meg:
        stages.append(("meg", ["om_gain", "-MEGadjoint", geom, cond, dip, "hm.bin", "h2mm.bin", "ds2mm.bin",
                               "meg.bin"]))
    for key, args in stages:
        _run(d, *args, threads=threads)
        if key in want:
            out[key] = io.read_bin(os.path.join(d, f"{key}.bin"))[1]
    import shutil
    shutil.rmtree(d, ignore_errors=True)
    return out

