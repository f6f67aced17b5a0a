"""Adjoint gradients of the gain against central finite differences.

L = sum(Gbar * G(sigma, dipoles)) for a fixed random cotangent Gbar; the
autograd gradients (DipSourceMat VJP kernel + conductivity adjoint reusing
the factorization) must match central differences with a step of 1e-6
(relative for conductivities) to 1e-5, and the mixed-precision gradient must
match the FP64 one.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(cuda, layers=3, inward=True):
    import torch
    from openmeeg_gb300 import api, workloads
    w = workloads.small(2, n_dipoles=6, layers=layers, inward=inward, perturb=True)
    geo = api.Geometry.from_head(w.head)
    sig0 = torch.tensor([d[2] for d in w.head.domains], dtype=torch.float64)
    dip0 = torch.as_tensor(w.dipoles, dtype=torch.float64, device=cuda)
    g = torch.Generator().manual_seed(3)
    k = w.electrodes.shape[0] + w.squids.shape[0]
    Gbar = torch.randn(k, w.dipoles.shape[0], generator=g, dtype=torch.float64).to(cuda)
    return w, geo, sig0, dip0, Gbar


def _loss(w, geo, sig, dip, Gbar, precision="fp64"):
    from openmeeg_gb300 import adjoint
    G = adjoint.gain(sig, dip, geo, w.head.domains, w.electrodes, w.squids, precision=precision)
    return (G * Gbar).sum()


@pytest.mark.parametrize("layers,inward", [(3, True), (4, False)])
def test_conductivity_gradient_matches_central_differences(cuda, layers, inward):
    import torch
    w, geo, sig0, dip0, Gbar = _setup(cuda, layers, inward)
    sig = sig0.clone().requires_grad_(True)
    L = _loss(w, geo, sig, dip0, Gbar)
    (gs,) = torch.autograd.grad(L, [sig])
    for kdom in range(len(sig0)):
        if sig0[kdom] == 0.0:
            assert gs[kdom] == 0.0
            continue
        h = 1e-6 * float(sig0[kdom])
        sp, sm = sig0.clone(), sig0.clone()
        sp[kdom] += h
        sm[kdom] -= h
        fd = (float(_loss(w, geo, sp, dip0, Gbar)) - float(_loss(w, geo, sm, dip0, Gbar))) / (2 * h)
        assert abs(float(gs[kdom]) - fd) <= 1e-5 * abs(fd), (kdom, float(gs[kdom]), fd)


def test_dipole_gradient_matches_central_differences(cuda):
    import torch
    w, geo, sig0, dip0, Gbar = _setup(cuda)
    dip = dip0.clone().requires_grad_(True)
    L = _loss(w, geo, sig0, dip, Gbar)
    (gd,) = torch.autograd.grad(L, [dip])
    gd = gd.cpu().numpy()
    fd = np.zeros_like(gd)
    for j in range(dip0.shape[0]):
        for c in range(6):
            h = 1e-6
            dp, dm = dip0.clone(), dip0.clone()
            dp[j, c] += h
            dm[j, c] -= h
            fd[j, c] = (float(_loss(w, geo, sig0, dp, Gbar)) - float(_loss(w, geo, sig0, dm, Gbar))) / (2 * h)
    assert np.linalg.norm(gd - fd) <= 1e-5 * np.linalg.norm(fd), np.abs(gd - fd).max()


def test_mixed_precision_gradient_matches_fp64(cuda):
    import torch
    w, geo, sig0, dip0, Gbar = _setup(cuda)
    out = {}
    for prec in ("fp64", "mixed"):
        sig = sig0.clone().requires_grad_(True)
        dip = dip0.clone().requires_grad_(True)
        L = _loss(w, geo, sig, dip, Gbar, precision=prec)
        out[prec] = [g.detach().cpu().numpy() for g in torch.autograd.grad(L, [sig, dip])]
    for a, b in zip(out["mixed"], out["fp64"]):
        assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b)
