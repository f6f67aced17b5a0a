"""The reference's own C++ API on the GB300 library (openmeeg_gb300/reference_shim).

The shim library defines OpenMEEG's HeadMat, SourceMatrix<Dipole>,
Head2EEGMat, Head2MEGMat, DipSource2MEGMat and SymMatrix::solveLin on top of
the C ABI; the reference's unmodified om_assemble and om_gain are relinked
with it ahead of the reference library.  These tests need the reference
sources (they compile against its headers) and run on the CPU:

* the shim exports the reference's symbols, and the relinked apps bind to it;
* without a GPU the relinked apps fail with the library's own error (their
  calls reach the GPU path, which fails loudly instead of running the CPU
  code);
* with OMG_SHIM_CPU_FALLBACK=1 every wrapped call hands over to the
  reference's implementation, and the outputs are the reference apps' own,
  byte for byte: the wrappers (and the geometry-file wrappers that run on
  every load) leave the reference's behaviour intact.
"""
import os
import subprocess

import pytest

from conftest import ROOT

SHIM = os.path.join(ROOT, "openmeeg_gb300", "reference_shim")
BIN = os.path.join(SHIM, "_build", "bin")


def _reference_dir():
    from oracle import ref_runner
    return ref_runner.REFERENCE_DIR


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    from oracle import ref_runner
    ref = _reference_dir()
    if not os.path.isdir(os.path.join(ref, "OpenMEEG", "include")):
        pytest.skip("reference sources absent")
    if not ref_runner.available():
        ref_runner.build()
    from openmeeg_gb300 import build
    build.build()
    subprocess.check_call(["make", "-s", "-C", SHIM, f"REF={ref}"], stdout=subprocess.DEVNULL)
    from openmeeg_gb300 import workloads
    d = str(tmp_path_factory.mktemp("shim"))
    w = workloads.small(1, layers=3)
    ref_runner.write_head(d, w.head, w.dipoles, w.electrodes, w.squids)
    return d


def _run(d, app, args, env=None, ref=False):
    """One app run; single-threaded, because the reference's DipSourceMat sums with OpenMP atomics, in an
    order (and so a last bit) that changes from run to run with several threads."""
    exe = os.path.join(ROOT, "oracle", "_ref", "bin", app) if ref else os.path.join(BIN, app)
    e = dict(os.environ)
    e["OMP_NUM_THREADS"] = "1"
    e.update(env or {})
    return subprocess.run([exe, *args], cwd=d, env=e, capture_output=True, text=True)


def test_shim_exports_the_reference_symbols(shim):
    out = subprocess.run(["nm", "-D", "--defined-only", "-C", os.path.join(SHIM, "_build", "libomg_refshim.so")],
                         capture_output=True, text=True, check=True).stdout
    for sym in ("OpenMEEG::HeadMat(OpenMEEG::Geometry const&, OpenMEEG::Integrator const&)",
                "OpenMEEG::Matrix OpenMEEG::SourceMatrix<OpenMEEG::Dipole>(",
                "OpenMEEG::Head2EEGMat(OpenMEEG::Geometry const&, OpenMEEG::Sensors const&)",
                "OpenMEEG::Head2MEGMat(OpenMEEG::Geometry const&, OpenMEEG::Sensors const&)",
                "OpenMEEG::DipSource2MEGMat(OpenMEEG::Matrix const&, OpenMEEG::Sensors const&)",
                "OpenMEEG::SymMatrix::solveLin(OpenMEEG::Matrix&) const",
                "OpenMEEG::Geometry::read_geometry_file("):
        assert sym in out, sym
    # the relinked apps load the shim ahead of the reference library
    ldd = subprocess.run(["ldd", os.path.join(BIN, "om_assemble")], capture_output=True, text=True).stdout
    assert ldd.index("libomg_refshim.so") < ldd.index("libomref.so")


@pytest.mark.skipif(os.path.exists("/dev/nvidia0"), reason="a GPU is present: the GPU tests cover the device path")
def test_shim_fails_loudly_without_a_gpu(shim):
    r = _run(shim, "om_assemble", ["-HM", "head.geom", "head.cond", "hm.bin"])
    assert r.returncode != 0
    assert "openmeeg_gb300" in r.stderr
    assert not os.path.exists(os.path.join(shim, "hm.bin"))


@pytest.mark.parametrize("app,args,out", [
    ("om_assemble", ["-HM", "head.geom", "head.cond"], "hm.bin"),
    ("om_assemble", ["-DSM", "head.geom", "head.cond", "dip.txt"], "dsm.bin"),
    ("om_assemble", ["-H2EM", "head.geom", "head.cond", "eeg.txt"], "h2em.bin"),
    ("om_assemble", ["-H2MM", "head.geom", "head.cond", "meg.txt"], "h2mm.bin"),
    ("om_assemble", ["-DS2MM", "dip.txt", "meg.txt"], "ds2mm.bin"),
])
def test_shim_hands_over_to_the_reference(shim, app, args, out):
    r = _run(shim, app, args + ["ref_" + out], ref=True)
    assert r.returncode == 0, r.stderr
    r = _run(shim, app, args + ["shim_" + out], env={"OMG_SHIM_CPU_FALLBACK": "1"})
    assert r.returncode == 0, r.stderr
    a = open(os.path.join(shim, "ref_" + out), "rb").read()
    b = open(os.path.join(shim, "shim_" + out), "rb").read()
    assert a == b


def test_shim_adjoint_gain_hands_over_to_the_reference(shim):
    for tag, env, ref in (("ref", None, True), ("shim", {"OMG_SHIM_CPU_FALLBACK": "1"}, False)):
        for app, args in (("om_assemble", ["-HM", "head.geom", "head.cond", f"{tag}_hm.bin"]),
                          ("om_assemble", ["-H2EM", "head.geom", "head.cond", "eeg.txt", f"{tag}_h2em.bin"]),
                          ("om_gain", ["-EEGadjoint", "head.geom", "head.cond", "dip.txt", f"{tag}_hm.bin",
                                       f"{tag}_h2em.bin", f"{tag}_geeg.bin"])):
            r = _run(shim, app, args, env=env, ref=ref)
            assert r.returncode == 0, r.stderr
    a = open(os.path.join(shim, "ref_geeg.bin"), "rb").read()
    b = open(os.path.join(shim, "shim_geeg.bin"), "rb").read()
    assert a == b
