"""GainEEG / GainMEG from an explicit inverse head matrix (om_minverser +
om_gain -EEG / -MEG, the pipeline of the reference's own tests) on the
library's kernels, against the reference's direct-form gains (golden fixture
direct_gains, made by tests/golden/make_golden.py).

Tolerances: relative Frobenius 1e-10 (FP64 products) and 1e-9 (the
FP64-accurate digit products on the tensor cores, mixed precision).
"""
import numpy as np
import pytest

from conftest import golden, rel

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "mixed": 1e-9}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("packed", [True, False])
def test_direct_gains_from_the_reference_inverse(cuda, precision, packed):
    """The reference's own packed inverse (om_minverser output) and its own
    source and sensor matrices: only the two products run here."""
    import torch
    from openmeeg_gb300 import api, io
    D = golden("direct_gains")
    G = golden("small_ico1_3l")
    Hp = D["hminv_packed_ico1_3l"]
    N = G["dsm"].shape[0]
    Hinv = Hp if packed else io.unpack_upper(Hp, N)
    ge = api.GainEEG(Hinv, G["dsm"], G["h2em"], precision=precision).cpu().numpy()
    gm = api.GainMEG(Hinv, G["dsm"], G["h2mm"], G["ds2mm"], precision=precision).cpu().numpy()
    assert rel(ge, D["eeg_ico1_3l"]) < TOL[precision]
    assert rel(gm, D["meg_ico1_3l"]) < TOL[precision]
    # the sparse sensor matrix given as a torch sparse tensor gives the same gain
    sp = torch.as_tensor(G["h2em"]).to_sparse()
    ge2 = api.GainEEG(Hinv, G["dsm"], sp, precision=precision).cpu().numpy()
    assert np.array_equal(ge, ge2)


@pytest.mark.parametrize("name", ["ico2_3l_pert", "config0"])
def test_direct_gains_on_library_matrices(cuda, name):
    """Every matrix from the library (FP64 drop-in), the inverse of its head
    matrix by LAPACK on the host, the gains on the GPU."""
    from openmeeg_gb300 import api, io, workloads
    D = golden("direct_gains")
    w = workloads.small(2, layers=3, perturb=True) if name == "ico2_3l_pert" else workloads.config0()
    geo = api.Geometry.from_head(w.head)
    HM = api.HeadMat(geo).cpu().numpy()
    Hinv = np.linalg.inv(HM)
    Hinv = 0.5 * (Hinv + Hinv.T)
    DSM = api.DipSourceMat(geo, w.dipoles)
    h2em = api.Head2EEGMat(geo, w.electrodes, sparse=True)
    H2MM = api.Head2MEGMat(geo, w.squids)
    DS2MM = api.DipSource2MEGMat(w.dipoles, w.squids)
    for precision in ("fp64", "mixed"):
        ge = api.GainEEG(io.packed_upper(Hinv), DSM, h2em, precision=precision).cpu().numpy()
        gm = api.GainMEG(Hinv, DSM, H2MM, DS2MM, precision=precision).cpu().numpy()
        assert rel(ge, D[f"eeg_{name}"]) < TOL[precision], precision
        assert rel(gm, D[f"meg_{name}"]) < TOL[precision], precision


def test_direct_gain_input_checks(cuda):
    from openmeeg_gb300 import api
    G = golden("small_ico1_3l")
    D = golden("direct_gains")
    Hp = D["hminv_packed_ico1_3l"]
    with pytest.raises(ValueError):
        api.GainEEG(Hp[:-1], G["dsm"], G["h2em"])             # not N(N+1)/2 entries
    with pytest.raises(ValueError):
        api.GainEEG(Hp, G["dsm"][:-1], G["h2em"])             # DSM rows != N
    import torch
    bad = (G["h2em"], torch.full((G["h2em"].shape[0], 3), 10 ** 6, dtype=torch.int64),
           torch.ones((G["h2em"].shape[0], 3), dtype=torch.float64))
    with pytest.raises(api.OMGError):
        api.GainEEG(Hp, G["dsm"], bad)                        # a column beyond N
    ge = api.GainEEG(Hp, G["dsm"][:, :0], G["h2em"])          # no dipoles
    assert ge.shape == (G["h2em"].shape[0], 0)
