"""Surface sources against the reference: SurfSourceMat and SurfSource2MEGMat
of a source icosphere in the brain of a 3-layer (inward meshes) and a 4-layer
(outward meshes) head, compared with the reference's om_assemble -SSM /
-SS2MM (tests/golden/surface_sources.npz) at 1e-12 relative Frobenius."""
import numpy as np
import pytest

from conftest import golden, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tag,layers,inward", [("3l", 3, True), ("4l_out", 4, False)])
def test_surface_source_matrices_match_reference(cuda, tag, layers, inward):
    from openmeeg_gb300 import api, workloads
    d = golden("surface_sources")
    w = workloads.small(1, layers=layers, inward=inward)
    geo = api.Geometry.from_head(w.head)
    A = api.SurfSourceMat(geo, d["src_vertices"], d["src_triangles"]).cpu().numpy()
    assert A.shape == d[f"ssm_{tag}"].shape
    assert rel(A, d[f"ssm_{tag}"]) <= 1e-12
    B = api.SurfSource2MEGMat(d["src_vertices"], d["src_triangles"], d[f"squids_{tag}"]).cpu().numpy()
    assert rel(B, d[f"ss2mm_{tag}"]) <= 1e-12


def test_source_mesh_crossing_an_interface_is_rejected(cuda):
    from openmeeg_gb300 import OMGError, api, workloads
    from openmeeg_gb300 import synthetic as syn
    w = workloads.small(1, layers=3)
    geo = api.Geometry.from_head(w.head)
    V, T = syn.icosphere(1, inward=False)
    with pytest.raises(OMGError, match="crosses an interface"):
        api.SurfSourceMat(geo, V * 0.3 + np.array([0.75, 0.0, 0.0]), T)   # straddles the inner surface (r = 0.87)
