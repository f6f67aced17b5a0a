"""The metric's own workloads on the GPU.

config1 (3 nested ico4 surfaces perturbed by a 2% spherical-harmonic field,
N = 17926, 64 EEG, 151 MEG): the mixed-precision gain against the FP64 drop-in
on all 2000 dipoles, and both against the reference's own ``om_gain
-EEGadjoint/-MEGadjoint`` output on the first 200 dipoles (golden fixture),
through the device entry point (omg_gain_dev) and the host one
(omg_gain_host).

config2 (the config1 geometry, 500 dipoles, conductivities sampled
log-uniformly within x[0.5, 2] of nominal): the autograd gradients of
L = sum(Gbar * [G_EEG; G_MEG]) with respect to the three conductivities and
the dipoles, FP64 and mixed, against central finite differences of the FP64
gain (relative step 1e-6 for the conductivities, absolute 1e-6 for the dipole
coordinates) to 1e-5, and the mixed gradient against the FP64 one to 1e-5.

Tolerances: FP64 gains 1e-10 against the reference, mixed gains 1e-6 against
FP64 and against the reference, gradients 1e-5.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden, rel

pytestmark = pytest.mark.gpu

TOL_GAIN = 1e-10
TOL_MIXED = 1e-6
TOL_GRAD = 1e-5


@pytest.fixture(scope="module")
def config1(cuda):
    from openmeeg_gb300 import api, workloads
    w = workloads.config1()
    geo = api.Geometry.from_head(w.head)
    ge, gm, st = api.forward_gain(geo, w.dipoles, w.electrodes, w.squids, precision="fp64")
    return w, geo, ge.cpu().numpy(), gm.cpu().numpy()


def test_config1_mixed_gain_device_entry_point(config1):
    from openmeeg_gb300 import api
    w, geo, ge64, gm64 = config1
    assert geo.size == 17926
    xe, xm, st = api.forward_gain(geo, w.dipoles, w.electrodes, w.squids, precision="mixed")
    xe, xm = xe.cpu().numpy(), xm.cpu().numpy()
    assert xe.shape == (64, 2000) and xm.shape == (151, 2000)
    assert rel(xe, ge64) < TOL_MIXED
    assert rel(xm, gm64) < TOL_MIXED
    assert st["refinement_steps"] >= 1


def test_config1_mixed_gain_host_entry_point(config1):
    from openmeeg_gb300 import api
    w, geo, ge64, gm64 = config1
    he, hm, _ = api.forward_gain(geo, w.dipoles, w.electrodes, w.squids, precision="mixed", host=True)
    assert isinstance(he, np.ndarray)
    assert rel(he, ge64) < TOL_MIXED
    assert rel(hm, gm64) < TOL_MIXED


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "config1_200.npz")), reason="config1 fixture absent")
@pytest.mark.parametrize("host", [False, True])
def test_config1_gains_match_reference_output(config1, host):
    from openmeeg_gb300 import api
    w, geo, ge64, gm64 = config1
    G = golden("config1_200")
    assert rel(ge64[:, :200], G["eeg"]) < TOL_GAIN
    assert rel(gm64[:, :200], G["meg"]) < TOL_GAIN
    xe, xm, _ = api.forward_gain(geo, w.dipoles[:200], w.electrodes, w.squids, precision="mixed", host=host)
    xe = xe if host else xe.cpu().numpy()
    xm = xm if host else xm.cpu().numpy()
    assert rel(xe, G["eeg"]) < TOL_MIXED
    assert rel(xm, G["meg"]) < TOL_MIXED


# ---------------------------------------------------------------------------
# config2: gradients
# ---------------------------------------------------------------------------
FD_DIPOLE_COORDS = 24     # dipole coordinates checked by central differences (of 500 x 6)


@pytest.fixture(scope="module")
def config2(cuda):
    import torch
    from openmeeg_gb300 import api, workloads
    w = workloads.config2()
    geo = api.Geometry.from_head(w.head)
    sig0 = torch.tensor([d[2] for d in w.head.domains], dtype=torch.float64)
    dip0 = torch.as_tensor(w.dipoles, dtype=torch.float64, device=cuda)
    k = w.electrodes.shape[0] + w.squids.shape[0]
    Gbar = torch.randn(k, w.dipoles.shape[0], generator=torch.Generator().manual_seed(5),
                       dtype=torch.float64).to(cuda)
    return w, geo, sig0, dip0, Gbar


def _loss(w, geo, sig, dip, Gbar, precision):
    from openmeeg_gb300 import adjoint
    G = adjoint.gain(sig, dip, geo, w.head.domains, w.electrodes, w.squids, precision=precision)
    return (G * Gbar).sum()


def _grads(w, geo, sig0, dip0, Gbar, precision):
    import torch
    sig = sig0.clone().requires_grad_(True)
    dip = dip0.clone().requires_grad_(True)
    L = _loss(w, geo, sig, dip, Gbar, precision)
    gs, gd = torch.autograd.grad(L, [sig, dip])
    return gs.detach().cpu().numpy(), gd.detach().cpu().numpy()


@pytest.fixture(scope="module")
def config2_grads(config2):
    w, geo, sig0, dip0, Gbar = config2
    return {p: _grads(w, geo, sig0, dip0, Gbar, p) for p in ("fp64", "mixed")}


def test_config2_conductivities_sampled_within_range(config2):
    from openmeeg_gb300 import workloads
    w, geo, sig0, dip0, Gbar = config2
    nominal = [d[2] for d in workloads.config1().head.domains]
    assert dip0.shape[0] == 500 and geo.size == 17926
    for s, s0 in zip(sig0.tolist(), nominal):
        if s0 == 0:
            assert s == 0
        else:
            assert 0.5 * s0 <= s <= 2.0 * s0 and s != s0


def test_config2_conductivity_gradient_matches_central_differences(config2, config2_grads):
    """Central differences of the FP64 gain, relative step 1e-6; both the FP64
    and the mixed-precision gradients must agree to 1e-5."""
    import torch
    w, geo, sig0, dip0, Gbar = config2
    fd = np.zeros(len(sig0))
    with torch.no_grad():
        for kd in range(len(sig0)):
            if sig0[kd] == 0.0:
                continue
            h = 1e-6 * float(sig0[kd])
            sp, sm = sig0.clone(), sig0.clone()
            sp[kd] += h
            sm[kd] -= h
            fd[kd] = (float(_loss(w, geo, sp, dip0, Gbar, "fp64")) - float(_loss(w, geo, sm, dip0, Gbar, "fp64"))) \
                / (2 * h)
    nz = sig0.numpy() > 0
    assert nz.sum() == 3
    for prec in ("fp64", "mixed"):
        gs = config2_grads[prec][0]
        assert np.all(gs[~nz] == 0.0)
        err = np.abs(gs[nz] - fd[nz]) / np.abs(fd[nz])
        assert err.max() <= TOL_GRAD, (prec, gs, fd)


def test_config2_dipole_gradient_matches_central_differences(config2, config2_grads):
    """Central differences over a seeded sample of dipole coordinates.  Column j
    of the gain depends only on dipole j and the head matrix does not depend on
    the dipoles, so each difference re-evaluates that one column,
    Y^T DSM(dipole j +- h) + DS2MM(dipole j +- h), with Y = HM^-1 [H2EM; H2MM]^T
    from the FP64 solver."""
    import torch
    from openmeeg_gb300 import api
    w, geo, sig0, dip0, Gbar = config2
    geo.set_conductivities(sig0.numpy())
    el, sq = w.electrodes, w.squids
    R = torch.cat([api.Head2EEGMat(geo, el), api.Head2MEGMat(geo, sq)], 0)      # k x N
    Y = api.Solver(geo, precision="fp64").solve(R.T.contiguous())                # N x k
    ne = el.shape[0]
    sq_d = torch.as_tensor(sq, dtype=torch.float64, device=dip0.device)

    def column_loss(d6, j):
        d = d6[None, :]
        g = (Y.T @ api.DipSourceMat(geo, d))[:, 0]
        g[ne:] += api.DipSource2MEGMat(d, sq_d)[:, 0]
        return float((g * Gbar[:, j]).sum())

    rng = np.random.default_rng(7)
    js = rng.choice(dip0.shape[0], FD_DIPOLE_COORDS, replace=False)
    cs = rng.integers(0, 6, FD_DIPOLE_COORDS)
    fd = np.zeros(FD_DIPOLE_COORDS)
    h = 1e-6
    for i, (j, c) in enumerate(zip(js, cs)):
        dp, dm = dip0[j].clone(), dip0[j].clone()
        dp[c] += h
        dm[c] -= h
        fd[i] = (column_loss(dp, j) - column_loss(dm, j)) / (2 * h)
    for prec in ("fp64", "mixed"):
        gd = config2_grads[prec][1][js, cs]
        assert np.linalg.norm(gd - fd) <= TOL_GRAD * np.linalg.norm(fd), (prec, np.abs(gd - fd).max())


def test_config2_mixed_gradient_matches_fp64(config2_grads):
    for a, b in zip(config2_grads["mixed"], config2_grads["fp64"]):
        assert np.linalg.norm(a - b) <= TOL_GRAD * np.linalg.norm(b)
