"""Differentiable forward gain: d(gain)/d(conductivities, dipoles).

The reference has no derivatives; this module adds them on top of the same
forward path.  With R the sensor rows ([Head2EEG; Head2MEG]), A = HeadMat,
D = DipSourceMat and the adjoint solution Y = A^-1 R^T (the one the gain
already computes), a cotangent Gbar of the gain G = R A^-1 D + [0; DS2MM]
pulls back as

* dipoles:  U = Y Gbar (N x n_dipoles); the DipSourceMat VJP kernel integrates
  the analytic derivatives of the dipole potential/gradient integrands
  against U over the forward's adaptive trees (omg_dipsourcemat_vjp_dev), plus
  the closed-form derivative of DS2MM;
* conductivities: Z = A^-1 (D Gbar^T) -- k extra solves on the same
  factorization -- and
      dL/dsigma_k = -tr(Y^T dA/dsigma_k Z) - (1/sigma_k) sum_{j in k} U_P0.D_P0
                    + sum_m o(k,m) tr(F_m Z_MEG).
  Every S block of A is proportional to its pair's coefficient
  K o sum(1/sigma), every N block (the deflated outermost block included) to
  K o sum(sigma) (OpenMEEG/src/assembleHeadMat.cpp:92-95, 27-60), so
  dA/dsigma_k is a block-wise rescaling of the assembled A; D blocks do not
  depend on sigma.  P0 rows of D carry 1/sigma of the dipole's domain
  (assembleSourceMat.cpp:94-96); MEG rows carry the conductivity jumps
  (assembleFerguson.cpp:25).

All contractions run on the library's GEMM kernel; torch holds the buffers.
"""
from __future__ import annotations

import ctypes
import math
from typing import Optional

import numpy as np
import torch

from . import _lib, api
from ._lib import MeshLayout, MeshPair, check

K = 1.0 / (4.0 * math.pi)
MAG = 1e-7


def _p(t: torch.Tensor, offset_elems: int = 0):
    return ctypes.c_void_p(t.data_ptr() + 8 * offset_elems)


class _Cols:
    """A column-major m x n FP64 matrix held as a (n, m) contiguous torch tensor."""

    def __init__(self, t: torch.Tensor):
        self.t = t
        self.m = t.shape[1]
        self.n = t.shape[0]


def _gemm(ctx, ta, tb, m, n, k, alpha, A, a_off, lda, B, b_off, ldb, beta, C, c_off, ldc):
    check(ctx.lib.omg_gemm_f64_dev(ctx.handle, ta, tb, m, n, k, alpha, _p(A, a_off), lda, _p(B, b_off), ldb, beta,
                                   _p(C, c_off), ldc))


def _layout(geo):
    info = geo.info()
    L = (MeshLayout * info.n_meshes)()
    check(geo.lib.omg_geometry_get_layout(geo.handle, info.n_meshes, L))
    n = ctypes.c_int32()
    check(geo.lib.omg_geometry_get_pairs(geo.handle, 0, None, ctypes.byref(n)))
    P = (MeshPair * n.value)()
    check(geo.lib.omg_geometry_get_pairs(geo.handle, n.value, P, ctypes.byref(n)))
    return list(L), list(P)


def _mesh_orientation(domains, orient, d, m):
    for b in domains[d][1]:
        if abs(b) - 1 == m:
            inside = b < 0
            return orient[m] if inside else -orient[m]
    return 0


def _common(domains, orient, m1, m2):
    d1 = {d for d in range(len(domains)) if _mesh_orientation(domains, orient, d, m1) != 0}
    d2 = {d for d in range(len(domains)) if _mesh_orientation(domains, orient, d, m2) != 0}
    return sorted(d1 & d2)


def ds2mm_torch(dipoles: torch.Tensor, squids: torch.Tensor) -> torch.Tensor:
    """DipSource2MEGMat in torch (assembleSensors.cpp:133-159), used only to
    differentiate the primary-field term (closed form, n_squids x n_dipoles)."""
    r, q = dipoles[:, :3], dipoles[:, 3:6]
    p, o = squids[:, :3], squids[:, 3:6]
    diff = p[:, None, :] - r[None, :, :]
    nd = torch.linalg.norm(diff, dim=2, keepdim=True)
    f = torch.cross(q[None, :, :].expand_as(diff), diff, dim=2) / nd ** 3
    return (f * o[:, None, :]).sum(2) * MAG / torch.linalg.norm(o, dim=1)[:, None]


class _Gain(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sigmas, dipoles, state):
        geo = state["geo"]
        lib_ctx = geo.ctx
        sig = sigmas.detach().double().cpu().numpy()
        geo.set_conductivities(sig)
        prec = state["precision"]
        dev = torch.device("cuda", lib_ctx.device)
        dip = dipoles.detach().to(dev, torch.float64).contiguous()
        el, sq = state["electrodes"], state["squids"]
        ne = 0 if el is None else el.shape[0]
        nm = 0 if sq is None else sq.shape[0]
        HM = api.HeadMat(geo, precision=prec).contiguous()                      # symmetric, N x N
        N = HM.shape[0]
        rows = []
        if ne:
            rows.append(api.Head2EEGMat(geo, el))
        if nm:
            rows.append(api.Head2MEGMat(geo, sq))
        Rm = torch.cat(rows, 0)                                                   # k x N
        sv = api.Solver(geo, precision=prec, hm=HM)
        Y = sv.solve(Rm.T.contiguous())                                           # N x k
        Yc = Y.T.contiguous()                                                     # column-major N x k
        D = api.DipSourceMat(geo, dip, integrator=state.get("dsm_integrator"))   # N x nd view
        Dc = D.T.contiguous()                                                     # column-major N x nd
        k, nd = Rm.shape[0], dip.shape[0]
        G = torch.empty((nd, k), dtype=torch.float64, device=dev)                 # column-major k x nd
        _gemm(lib_ctx, 1, 0, k, nd, N, 1.0, Yc, 0, N, Dc, 0, N, 0.0, G, 0, k)
        G = G.T.contiguous()                                                      # k x nd row-major
        if nm:
            G[ne:] += api.DipSource2MEGMat(dip, sq, lib_ctx)
        state.update(dict(HM=HM, Yc=Yc, Dc=Dc, sv=sv, dip=dip, N=N, ne=ne, nm=nm, sig=sig))
        ctx.state = state
        ctx.in_devices = (sigmas.device, sigmas.dtype, dipoles.device, dipoles.dtype)
        return G

    @staticmethod
    def backward(ctx, Gbar):
        st = ctx.state
        geo, lib_ctx = st["geo"], st["geo"].ctx
        HM, Yc, Dc, sv, dip = st["HM"], st["Yc"], st["Dc"], st["sv"], st["dip"]
        N, ne, nm, sig = st["N"], st["ne"], st["nm"], st["sig"]
        k, nd = Yc.shape[0], Dc.shape[0]
        dev = HM.device
        Gb = Gbar.detach().to(dev, torch.float64).contiguous()                   # k x nd
        Gbc = Gb.T.contiguous()                                                   # column-major k x nd
        # U = Y Gbar (N x nd), column-major
        U = torch.empty((nd, N), dtype=torch.float64, device=dev)
        _gemm(lib_ctx, 0, 0, N, nd, k, 1.0, Yc, 0, N, Gbc, 0, k, 0.0, U, 0, N)
        # ---- dipoles
        ddip = torch.zeros((nd, 6), dtype=torch.float64, device=dev)
        it = _lib.Integrator(3, 10, 0.001) if st.get("dsm_integrator") is None else st["dsm_integrator"]
        check(lib_ctx.lib.omg_dipsourcemat_vjp_dev(lib_ctx.handle, geo.handle, _p(dip), nd, ctypes.byref(it), -1,
                                                   _p(U), N, _p(ddip)))
        if nm:
            d = dip.detach().clone().requires_grad_(True)
            with torch.enable_grad():
                v = (ds2mm_torch(d, st["squids"]) * Gb[ne:]).sum()
            ddip = ddip + torch.autograd.grad(v, d)[0]
        # ---- conductivities
        W = torch.empty((k, N), dtype=torch.float64, device=dev)                  # D Gbar^T, column-major N x k
        _gemm(lib_ctx, 0, 1, N, k, nd, 1.0, Dc, 0, N, Gbc, 0, k, 0.0, W, 0, N)
        Z = sv.solve(W.T.contiguous())                                            # N x k
        Zc = Z.T.contiguous()
        layout, pairs = _layout(geo)
        domains = st["domains"]
        orient = [m.orientation for m in layout]
        nv = layout[-1].vend if layout else 0

        def rows_of(m, kind):
            L = layout[m]
            if kind == "V":
                return L.vbeg, L.vend
            return (L.tri_unknown, L.tri_unknown + L.n_triangles) if L.tri_unknown >= 0 else None

        def trace(r, c):
            """tr(Y[r]^T A[r, c] Z[c]) with A the symmetric head matrix."""
            (r0, r1), (c0, c1) = r, c
            P = torch.empty((k, r1 - r0), dtype=torch.float64, device=dev)
            _gemm(lib_ctx, 0, 0, r1 - r0, k, c1 - c0, 1.0, HM, r0 + c0 * N, N, Zc, c0, N, 0.0, P, 0, r1 - r0)
            return float((P * Yc[:, r0:r1]).sum())

        ndom = len(domains)
        grad_sigma = np.zeros(ndom)
        for pr in pairs:
            common = _common(domains, orient, pr.m1, pr.m2)
            blocks = []
            # S block: present in A for pairs without a current barrier
            s1, s2 = rows_of(pr.m1, "T"), rows_of(pr.m2, "T")
            if s1 is not None and s2 is not None:
                blocks.append(("S", s1, s2, pr.cS))
            blocks.append(("N", rows_of(pr.m1, "V"), rows_of(pr.m2, "V"), pr.cN))
            for kind, r, c, coef in blocks:
                t = trace(r, c) + (trace(c, r) if pr.m1 != pr.m2 else 0.0)
                for dk in common:
                    if kind == "S":
                        dc = -pr.orientation * K / sig[dk] ** 2
                    else:
                        dc = pr.orientation * K
                    grad_sigma[dk] -= (dc / coef) * t
        # P0 rows of D scale with 1/sigma of the dipole's domain
        dom = torch.empty(nd, dtype=torch.int32, device=dev)
        check(lib_ctx.lib.omg_dipole_domains_dev(lib_ctx.handle, geo.handle, _p(dip), nd, ctypes.c_void_p(dom.data_ptr())))
        domh = dom.cpu().numpy()
        for dk in range(ndom):
            js = np.nonzero(domh == dk)[0]
            if len(js) == 0 or sig[dk] == 0.0:
                continue
            acc = 0.0
            for b in domains[dk][1]:
                rr = rows_of(abs(b) - 1, "T")
                if rr is None:
                    continue
                jj = torch.as_tensor(js, device=dev)
                acc += float((U[jj, rr[0]:rr[1]] * Dc[jj, rr[0]:rr[1]]).sum())
            grad_sigma[dk] -= acc / sig[dk]
        # MEG rows carry the conductivity jumps: H2MM = sum_m jump_m F_m
        if nm:
            sq = st["squids"]
            for m in range(len(layout)):
                F = torch.empty((N, nm), dtype=torch.float64, device=dev)         # column-major nm x N
                check(lib_ctx.lib.omg_head2megmat_mesh_dev(lib_ctx.handle, geo.handle, _p(sq), nm, m, _p(F)))
                t = float((F * Zc[ne:, :].T).sum())                               # sum_i F[i,:] . Z[:, ne+i]
                for dk in range(ndom):
                    o = _mesh_orientation(domains, orient, dk, m)
                    if o:
                        grad_sigma[dk] += o * t
        # a zero conductivity (air) fixes the structure of the system (no
        # potential-jump unknowns outside); it is not a parameter
        grad_sigma[np.asarray(sig) == 0.0] = 0.0
        sdev, sdt, ddev, ddt = ctx.in_devices
        gs = torch.as_tensor(grad_sigma, dtype=sdt, device=sdev)
        return gs, ddip.to(ddev, ddt), None


def gain(sigmas: torch.Tensor, dipoles: torch.Tensor, geo: "api.Geometry", domains, electrodes=None, squids=None,
         precision: str = "fp64", dsm_integrator: Optional[_lib.Integrator] = None) -> torch.Tensor:
    """Differentiable gain [EEG; MEG] (k x n_dipoles) as a function of the
    domain conductivities (geometry domain order) and the dipoles (n x 6).

    `domains` is the geometry's .geom-style domain list
    [(name, [signed 1-based interface ids], sigma), ...]; its sigmas are
    replaced by `sigmas`.  Conductivities set to zero (e.g. air) must stay
    zero; their gradient is returned as 0.
    """
    dev = torch.device("cuda", geo.ctx.device)
    el = None if electrodes is None else torch.as_tensor(np.asarray(electrodes)[:, :3], dtype=torch.float64,
                                                         device=dev).contiguous()
    sq = None if squids is None else torch.as_tensor(np.asarray(squids)[:, :6], dtype=torch.float64,
                                                     device=dev).contiguous()
    state = {"geo": geo, "electrodes": el, "squids": sq, "precision": precision, "domains": domains,
             "dsm_integrator": dsm_integrator}
    return _Gain.apply(sigmas, dipoles, state)
