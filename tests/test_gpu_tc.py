"""The tcgen05 tensor-core GEMM (3xTF32 split) against an FP64 torch product.

C = beta*C + alpha*A*B^T with A (M x K) and B (N x K) K-major, split into
TF32 heads and FP32 remainders.  Tolerances: 3-term split 1e-5 (FP32-level),
head-only product 5e-3 (TF32-level), relative Frobenius.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _split(x):
    import torch
    h = (x.view(torch.int32) & ~0x1FFF).view(torch.float32)
    return h.contiguous(), (x - h).contiguous()


def _lib():
    from openmeeg_gb300 import _lib
    lib = _lib.load()
    f = lib.omg_internal_gemm_tf32x3
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p,
                  ctypes.c_int64, ctypes.c_int, ctypes.c_void_p]
    return f


def _run(M, N, K, alpha, beta, lower, three, seed=0):
    import torch
    f = _lib()
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.randn(M, K, device="cuda", generator=g, dtype=torch.float32)
    B = A if lower else torch.randn(N, K, device="cuda", generator=g, dtype=torch.float32)
    Ah, Al = _split(A)
    Bh, Bl = _split(B)
    C0 = torch.randn(N, M, device="cuda", generator=g, dtype=torch.float32)   # column-major M x N
    C = C0.clone()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)
    rc = f(M, N, K, alpha, p(Ah), p(Al if three else None), K, p(Bh), p(Bl if three else None), K, beta, p(C), M,
           1 if lower else 0, p(err))
    assert rc == 0 and int(err.item()) == 0
    ref = (beta * C0.double().T + alpha * (A.double() @ B.double().T))
    got = C.double().T
    if lower:
        mask = torch.tril(torch.ones(M, N, dtype=torch.bool, device="cuda"))
        # entries above the diagonal are untouched
        assert torch.equal(got[~mask], C0.double().T[~mask])
        ref, got = ref[mask], got[mask]
    return float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))


@pytest.mark.parametrize("M,N,K", [(128, 128, 32), (300, 200, 128), (1000, 215, 96)])
def test_tc_gemm_3xtf32_general(cuda, M, N, K):
    assert _run(M, N, K, 1.0, 0.0, False, True) < 1e-5
    assert _run(M, N, K, -1.0, 1.0, False, True) < 1e-5


def test_tc_gemm_head_only_is_tf32_accurate(cuda):
    e = _run(256, 256, 128, 1.0, 0.0, False, False)
    assert 1e-6 < e < 5e-3


def test_tc_gemm_lower_update(cuda):
    assert _run(640, 640, 128, -1.0, 1.0, True, True) < 1e-5


@pytest.mark.parametrize("M,N,K,row0", [(1000, 128, 128, 0), (777, 90, 128, 128), (4300, 128, 96, 40)])
def test_tc_gemm_epilogue_split_copy(cuda, M, N, K, row0):
    """The epilogue's K-major TF32 head/remainder copy of C's rows >= row0 (row
    stride 128, zero past N) equals the split of the C it writes, bit for bit."""
    import torch
    from openmeeg_gb300 import _lib
    f = _lib.load().omg_internal_gemm_tf32x3_split
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p,
                  ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
    g = torch.Generator(device="cuda").manual_seed(M)
    A = torch.randn(M, K, device="cuda", generator=g)
    B = torch.randn(N, K, device="cuda", generator=g)
    Ah, Al = _split(A)
    Bh, Bl = _split(B)
    C = torch.randn(N, M, device="cuda", generator=g)          # column-major M x N
    Sh = torch.full((M - row0, 128), 7.0, device="cuda")         # garbage that must be overwritten
    Sl = torch.full((M - row0, 128), 7.0, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert f(M, N, K, -1.0, p(Ah), p(Al), K, p(Bh), p(Bl), K, 1.0, p(C), M, p(Sh), p(Sl), row0, p(err)) == 0
    assert int(err.item()) == 0
    rows = C.T[row0:]                                            # (M - row0) x N, row-major
    h, l = _split(rows.contiguous())
    assert torch.equal(Sh[:, :N], h) and torch.equal(Sl[:, :N], l)
    assert float(Sh[:, N:].abs().max() if N < 128 else 0.0) == 0.0 and float(Sl[:, N:].abs().max() if N < 128 else 0.0) == 0.0


def _epi_hook():
    return _lib_hook("omg_internal_gemm_tf32x3_epi",
                     [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p,
                      ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                      ctypes.c_float, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                      ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p])


@pytest.mark.parametrize("M,N,K", [(128, 128, 128), (700, 300, 96), (17000, 215, 128)])
def test_tc_gemm_epilogue_head_remainder(cuda, M, N, K):
    """C written as TF32 heads with the remainders in Cr: Ch + Cr is the
    3xTF32 product, and the pair is the exact split of that sum."""
    import torch
    f = _epi_hook()
    g = torch.Generator(device="cuda").manual_seed(N)
    A = torch.randn(M, K, device="cuda", generator=g)
    B = torch.randn(N, K, device="cuda", generator=g)
    Ah, Al = _split(A)
    Bh, Bl = _split(B)
    C = torch.full((N, M), 3.0, device="cuda")                   # column-major M x N, overwritten (beta = 0)
    Cr = torch.full((N, M), 3.0, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)
    assert f(M, N, K, 1.0, p(Ah), p(Al), K, p(Bh), p(Bl), K, 0.0, p(C), M, p(Cr), None, None, 0, p(err)) == 0
    assert int(err.item()) == 0
    v = C + Cr
    h, l = _split(v.contiguous())
    assert torch.equal(h, C) and torch.equal(l, Cr)
    ref = A.double() @ B.double().T
    assert float(torch.linalg.norm(v.double().T - ref) / torch.linalg.norm(ref)) < 1e-5
    # beta != 0 with a remainder output is refused
    assert f(M, N, K, 1.0, p(Ah), p(Al), K, p(Bh), p(Bl), K, 1.0, p(C), M, p(Cr), None, None, 0, p(err)) == -1


@pytest.mark.parametrize("M,N,K,row0", [(1000, 215, 128, 0), (1000, 215, 128, 384), (90, 300, 64, 0),
                                        (4096, 64, 128, 3968)])
def test_tc_gemm_epilogue_band_copy(cuda, M, N, K, row0):
    """The transposed band copy: row j of Xh/Xl (stride 128) is the TF32 split
    of column j of C's rows row0 .. row0+127, zero at rows past M."""
    import torch
    f = _epi_hook()
    g = torch.Generator(device="cuda").manual_seed(M + row0)
    A = torch.randn(M, K, device="cuda", generator=g)
    B = torch.randn(N, K, device="cuda", generator=g)
    Ah, Al = _split(A)
    Bh, Bl = _split(B)
    C = torch.randn(N, M, device="cuda", generator=g)            # column-major M x N
    Xh = torch.full((N, 128), 7.0, device="cuda")                # garbage that must be overwritten
    Xl = torch.full((N, 128), 7.0, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)
    assert f(M, N, K, -1.0, p(Ah), p(Al), K, p(Bh), p(Bl), K, 1.0, p(C), M, None, p(Xh), p(Xl), row0, p(err)) == 0
    assert int(err.item()) == 0
    rows = min(128, M - row0)
    band = C[:, row0:row0 + rows].contiguous()                   # N x rows: column j of the band as row j
    h, l = _split(band)
    assert torch.equal(Xh[:, :rows], h) and torch.equal(Xl[:, :rows], l)
    if rows < 128:
        assert float(Xh[:, rows:].abs().max()) == 0.0 and float(Xl[:, rows:].abs().max()) == 0.0
    # a band that does not start on a tile row is refused
    assert f(M, N, K, -1.0, p(Ah), p(Al), K, p(Bh), p(Bl), K, 1.0, p(C), M, None, p(Xh), p(Xl), 8, p(err)) == -1


@pytest.mark.parametrize("M,N,K,lower", [(5000, 1000, 64, False), (4100, 4100, 128, True)])
def test_tc_gemm_many_tiles_per_cta(cuda, M, N, K, lower):
    # more tiles than SMs: every CTA walks several tiles through both TMEM accumulators
    assert _run(M, N, K, -1.0, 1.0, lower, True) < 1e-5


def _lib_hook(name, argtypes):
    from openmeeg_gb300 import _lib
    f = getattr(_lib.load(), name)
    f.restype = ctypes.c_int
    f.argtypes = argtypes
    return f


def _residual_hook():
    from openmeeg_gb300 import _lib
    f = _lib.load().omg_internal_residual_tc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int64, ctypes.c_int64] + [ctypes.c_void_p] * 5
    return f


@pytest.mark.parametrize("n,k", [(300, 7), (2500, 215), (4486, 130)])
def test_tc_residual_is_fp64_accurate(cuda, n, k):
    """R = B - A X from bf16 digits with exact windowed accumulation.  Digit
    truncation (7 digits of 7 bits per row / column scale, levels <= 8) leaves
    errors near 2^-48 of n times the row and column maxima: below 5e-13
    normwise relative to |A||X| and 1e-10 elementwise even with entries spread
    over 1e5 in a row; an inexact tensor-core sum would show up near 1e-7."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(n + k)
    M = torch.randn(n, n, device="cuda", dtype=torch.float64, generator=g)
    # entries over several orders of magnitude, symmetric, strong diagonal
    scale = torch.exp(torch.randn(n, device="cuda", dtype=torch.float64, generator=g) * 2)
    A = (M + M.T) * scale[:, None] * scale[None, :] + torch.diag(scale ** 2 * n)
    X = torch.randn(n, k, device="cuda", dtype=torch.float64, generator=g) * 10.0 ** torch.randint(
        -3, 4, (1, k), device="cuda", generator=g)
    B = A @ X + 1e-7 * torch.randn(n, k, device="cuda", dtype=torch.float64, generator=g) * (A.abs() @ X.abs())
    Xc, Bc = X.T.contiguous(), B.T.contiguous()          # column-major n x k
    Rc = torch.empty_like(Bc)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert _residual_hook()(n, k, p(A), p(Xc), p(Bc), p(Rc), p(err)) == 0 and int(err.item()) == 0
    R = Rc.T
    ref = B - A @ X
    scale_ax = A.abs() @ X.abs()
    elem = float(((R - ref).abs() / scale_ax).max())
    norm = float(torch.linalg.norm(R - ref) / torch.linalg.norm(scale_ax))
    assert elem < 1e-10 and norm < 5e-13, (elem, norm)


def _digits_ref(col, nd, beta, ldo):
    """Digit rows of one column as the kernel defines them: e = frexp exponent
    of the largest magnitude, Y = x 2^(nd beta - e) rounded half to even, then
    balanced base-2^beta digits from the lowest up (plane 0 takes the rest)."""
    m = float(np.max(np.abs(col))) if col.size else 0.0
    e = int(np.frexp(m)[1])
    Y = [int(v) for v in np.rint(np.ldexp(col, nd * beta - e))]   # exact: power-of-two scaling, rint ties to even
    Y += [0] * (ldo - len(Y))
    planes = np.zeros((nd, ldo))
    half, mask = 1 << (beta - 1), (1 << beta) - 1
    for d in range(nd - 1, 0, -1):
        r = [((y + half) & mask) - half for y in Y]
        planes[d] = r
        Y = [(y - ri) >> beta for y, ri in zip(Y, r)]
    planes[0] = Y
    return planes, e


@pytest.mark.parametrize("nd", [7, 6])
def test_digit_planes_bit_exact(cuda, nd):
    """The digit planes and column exponents of the integer-arithmetic digit
    kernel equal the definition evaluated in exact integers: columns with zero,
    signed zeros, subnormals, exact ties of the rounding and entries over 600
    binary orders; n not a multiple of 4; padding rows and columns zero.  Six
    digits of base 2^7 (the library's layout) take the kernel compiled for that
    layout, seven the general one."""
    import torch
    f = _lib_hook("omg_internal_digits", [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_int64,
                                          ctypes.c_void_p, ctypes.c_void_p])
    rng = np.random.default_rng(5)
    n, ncol, ldm, beta = 301, 9, 305, 7
    ldo, rpp = 320, 12
    M = np.zeros((ncol, ldm))
    M[0, :n] = rng.standard_normal(n)
    M[1, :n] = rng.standard_normal(n) * np.exp2(rng.integers(-300, 300, n).astype(float))
    M[2, :n] = 0.0
    M[2, 5] = -0.0
    M[3, :n] = rng.standard_normal(n) * 1e-310                      # subnormal column
    M[4, :n] = rng.standard_normal(n)
    M[4, 0] = 1.0
    tie = np.exp2(-(nd * beta - 1))                                  # the digit grid's step (column max 1)
    M[4, 1:20] = (np.arange(19) + 0.5) * tie                          # exact ties of the digit grid
    M[4, 20:40] = -(np.arange(20) + 0.5) * tie
    M[5, :n] = -rng.random(n) * 3e8
    M[6, :n] = rng.standard_normal(n)
    M[6, 7] = -4.0                                                   # the largest magnitude negative
    M[7, :n] = np.exp2(rng.integers(-60, 0, n).astype(float))
    M[8, :n] = rng.standard_normal(n) * 1e-3
    Md = torch.tensor(M, device="cuda", dtype=torch.float64)
    out = torch.full((nd * rpp * ldo,), 7, dtype=torch.int16, device="cuda")   # garbage to be overwritten
    ex = torch.zeros(rpp, dtype=torch.int32, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert f(p(Md), n, ncol, ldm, nd, beta, rpp, ldo, p(out), p(ex)) == 0
    got = out.view(torch.bfloat16).float().cpu().numpy().reshape(nd, rpp, ldo)
    exg = ex.cpu().numpy()
    for c in range(ncol):
        ref, e = _digits_ref(M[c, :n], nd, beta, ldo)
        assert exg[c] == e, (c, exg[c], e)
        assert np.array_equal(got[:, c, :], ref), c
    assert not got[:, ncol:, :].any()
    # layouts the 8-byte stores cannot take are refused
    assert f(p(Md), n, ncol, ldm, nd, beta, rpp, 302, p(out), p(ex)) == -1


def test_diagonal_block_cholesky_and_inverse(cuda):
    """One CTA factors a 128 x 128 SPD block and inverts the factor:
    L L^T = A and L Linv = I at FP32 level; the K-major split of Linv adds
    back to Linv; a partial block (n = 77) leaves zero padding."""
    import torch
    f = _lib_hook("omg_internal_potrf_inv", [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                             ctypes.c_void_p] + [ctypes.c_void_p] * 4)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    none4 = [None] * 4
    for n in (128, 77):
        g = torch.Generator(device="cuda").manual_seed(n)
        M = torch.randn(n, n, device="cuda", dtype=torch.float64, generator=g)
        A64 = M @ M.T / n + torch.eye(n, device="cuda", dtype=torch.float64)
        A = torch.zeros(140, 140, device="cuda", dtype=torch.float32)   # column-major, lda = 140
        A[:n, :n] = A64.T.float()
        Li = torch.zeros(128 * 128, device="cuda")
        Bh = torch.zeros(128 * 128, device="cuda")
        Bl = torch.zeros(128 * 128, device="cuda")
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        us = ctypes.c_float(0)
        assert f(n, p(A), 140, p(Li), p(Bh), p(Bl), p(err), 20, ctypes.byref(us), *none4) == 0
        assert int(err.item()) == 0
        print(f"potrf_inv n={n}: {us.value:.1f} us per launch")
        L = torch.tril(A.T[:n, :n].double())            # row-major view of the factor
        assert float(torch.linalg.norm(L @ L.T - A64) / torch.linalg.norm(A64)) < 1e-6
        Linv = Li.view(128, 128).T.double()               # stored column-major
        assert float(torch.linalg.norm(L @ Linv[:n, :n] - torch.eye(n, device="cuda", dtype=torch.float64))) < 1e-5
        if n < 128:
            assert float(Linv[n:, :].abs().max()) == 0.0 and float(Linv[:, n:].abs().max()) == 0.0
        assert torch.equal((Bh + Bl).view(128, 128), Li.view(128, 128).T)


def test_diagonal_block_panel_update(cuda):
    """The diagonal-block update applies A11 -= P0 P0^T + P1 P1^T from the
    head / remainder rows of one or two panels (n rows of 128 values) before
    the block is factored: L L^T equals the updated block at FP32 level (full
    and partial blocks), and nothing outside the n x n block is written."""
    import torch
    f = _lib_hook("omg_internal_potrf_inv", [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                             ctypes.c_void_p] + [ctypes.c_void_p] * 4)
    p = lambda t: ctypes.c_void_p(t.data_ptr())

    def split(P):
        h = (P.view(torch.int32) & -8192).view(torch.float32)   # TF32 head: low 13 mantissa bits cleared
        return h.contiguous(), (P - h).contiguous()

    for n, npanels in ((128, 2), (128, 1), (77, 2)):
        g = torch.Generator(device="cuda").manual_seed(1000 + n + npanels)
        M = torch.randn(n, n, device="cuda", dtype=torch.float64, generator=g)
        Af = M @ M.T / n + torch.eye(n, device="cuda", dtype=torch.float64)   # the block after the update
        Ps = [torch.randn(n, 128, device="cuda", generator=g).mul_(0.1) for _ in range(npanels)]
        Ain = Af.clone()
        for P in Ps:
            Ain += P.double() @ P.double().T
        A = torch.zeros(140, 140, device="cuda", dtype=torch.float32)
        A[:n, :n] = Ain.T.float()
        Li = torch.zeros(128 * 128, device="cuda")
        Bh = torch.zeros(128 * 128, device="cuda")
        Bl = torch.zeros(128 * 128, device="cuda")
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        hl = [split(P) for P in Ps]
        args = [p(t) for pair in hl for t in pair] + [None] * (4 - 2 * len(hl))
        us = ctypes.c_float(0)
        assert f(n, p(A), 140, p(Li), p(Bh), p(Bl), p(err), 20, ctypes.byref(us), *args) == 0
        assert int(err.item()) == 0
        print(f"potrf_inv n={n} with {npanels} panel update(s): {us.value:.1f} us per launch")
        L = torch.tril(A.T[:n, :n].double())
        assert float(torch.linalg.norm(L @ L.T - Af) / torch.linalg.norm(Af)) < 2e-6
        Linv = Li.view(128, 128).T.double()
        assert float(torch.linalg.norm(L @ Linv[:n, :n] - torch.eye(n, device="cuda", dtype=torch.float64))) < 1e-5
        assert float(A[n:, :].abs().max()) == 0.0 and float(A[:, n:].abs().max()) == 0.0


@pytest.mark.parametrize("nrhs", [1, 215, 300])
@pytest.mark.parametrize("name", ["ico2", "config0"])
def test_persistent_sweep_solve(cuda, name, nrhs, monkeypatch):
    """The mixed solver's triangular sweeps as one persistent launch each
    (tiles of 64 right-hand sides claimed in dependency order, flags between
    them) against the chain of one tensor-core update per block, and against a
    dense FP64 solve; 215 and 300 right-hand sides take 4 and 5 column groups."""
    from openmeeg_gb300 import api, workloads
    w = workloads.small(2, layers=3, perturb=True) if name == "ico2" else workloads.config0()
    geo = api.Geometry.from_head(w.head)
    HM = api.HeadMat(geo, precision="mixed").cpu().numpy()
    rng = np.random.default_rng(nrhs)
    B = rng.standard_normal((HM.shape[0], nrhs))
    sv = api.Solver(geo, precision="mixed")
    X = sv.solve(B).cpu().numpy()
    monkeypatch.setenv("OMG_SOLVE_CHAIN", "1")
    Xc = sv.solve(B).cpu().numpy()
    monkeypatch.delenv("OMG_SOLVE_CHAIN")
    ref = np.linalg.solve(HM, B)
    # both stop refining once the predicted error is below the solver's tolerance, 1e-6
    e_sweep = np.linalg.norm(X - ref) / np.linalg.norm(ref)
    e_chain = np.linalg.norm(Xc - ref) / np.linalg.norm(ref)
    assert e_sweep <= 1e-6 and e_chain <= 1e-6, (e_sweep, e_chain)
    X2 = sv.solve(B).cpu().numpy()          # flags and counters are reset for every sweep
    assert np.array_equal(X, X2)


@pytest.mark.parametrize("name", ["ico2", "config0"])
def test_grouped_fold_matches_separate_launches(cuda, name, monkeypatch):
    """The folds of the diagonal-block inverses into the solve operators
    (W_b <- L21_b Linv_b and block row b <- Linv_b x block row b) run as one
    grouped persistent launch; one launch per product (OMG_FOLD_SEPARATE=1)
    computes every tile the same way, so the factors, and the solutions, are
    bit-identical."""
    from openmeeg_gb300 import api, workloads
    w = workloads.small(2, layers=3, perturb=True) if name == "ico2" else workloads.config0()
    geo = api.Geometry.from_head(w.head)
    rng = np.random.default_rng(7)
    B = rng.standard_normal((geo.size, 37))
    X = api.Solver(geo, precision="mixed").solve(B).cpu().numpy()
    monkeypatch.setenv("OMG_FOLD_SEPARATE", "1")
    Xs = api.Solver(geo, precision="mixed").solve(B).cpu().numpy()
    monkeypatch.delenv("OMG_FOLD_SEPARATE")
    assert np.isfinite(X).all()
    assert np.array_equal(X, Xs)
