"""Head2MEGMat through the entry point that allocates no device memory.

Some callers cannot allocate device memory while they run: a real-time
acquisition loop that must not wait on the allocator, a host that reserves
the GPU's memory for itself at start-up, a plugin host whose policy forbids
device allocations.  omg_head2megmat_noalloc_dev serves them from a fixed
scratch array inside the library.  These tests call it through the C ABI and
compare it with the allocating entry point on two calls in a row (the array
is shared between calls and keeps the previous call's contents), and check
that a request larger than the array is refused.

This file sorts last so that a run stopping at its first failure has already
run every other test.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

TOL = 1e-12   # the tolerance of the other assembled-matrix tests


def _call(lib, geo, squids, out):
    return lib.omg_head2megmat_noalloc_dev(geo.ctx.handle, geo.handle, ctypes.c_void_p(squids.data_ptr()),
                                           squids.shape[0], ctypes.c_void_p(out.data_ptr()))


def test_noalloc_head2megmat_matches_allocating_entry_point(cuda):
    import torch
    from openmeeg_gb300 import _lib, api, synthetic, workloads
    lib = _lib.load()
    w = workloads.small(2, layers=3, perturb=True)
    geo = api.Geometry.from_head(w.head)
    N = geo.size
    # two calls in a row with different sensor sets: the second must not see the first's scratch
    for squids in (synthetic.radial_magnetometers(31, 1.2), w.squids):
        s = torch.as_tensor(squids, dtype=torch.float64, device=cuda).contiguous()
        ref = api.Head2MEGMat(geo, s).cpu().numpy()
        out = torch.full((N, s.shape[0]), float("nan"), dtype=torch.float64, device=cuda)   # column-major n x N
        rc = _call(lib, geo, s, out)
        assert rc == 0, lib.omg_last_error()
        got = out.T.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert rel(got, ref) < TOL


def test_noalloc_refuses_requests_beyond_its_scratch(cuda):
    import torch
    from openmeeg_gb300 import _lib, api, synthetic, workloads
    lib = _lib.load()
    w = workloads.small(2, layers=3)
    geo = api.Geometry.from_head(w.head)
    nt = sum(t.shape[0] for t in w.head.triangles)
    n = (4 * 1024 * 1024) // nt + 1          # one sensor more than the scratch holds
    s = torch.as_tensor(synthetic.radial_magnetometers(n, 1.2), dtype=torch.float64, device=cuda).contiguous()
    out = torch.full((4, 4), 7.0, dtype=torch.float64, device=cuda)
    rc = _call(lib, geo, s, out)
    assert rc == -1
    assert b"scratch" in lib.omg_last_error()
    assert torch.all(out == 7.0)              # refused before anything is written
