"""On-device uniform mesh refinement against the host generator: the same
vertex and face numbering, positions bitwise equal, areas to the last bits of
tan/atan, the same parent/leaf slot structure."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,level", [(1, 0), (1, 1), (1, 4), (1, 6), (2, 1), (2, 5), (3, 1),
                                        (3, 6)])
def test_device_mesh_matches_host(gpu_ctx, kind, level):
    import torch

    from lpm_gb300 import core

    radius = 4.0 if kind == core.MESH_QUAD_RECT else 1.0
    hv, hf, ha, hm = core.build_mesh(kind, level, radius)
    dv, df, da, dmask = core.build_mesh_device(gpu_ctx, kind, level, radius)
    torch.cuda.synchronize()
    assert np.array_equal(dv.cpu().numpy(), hv)
    assert np.array_equal(df.cpu().numpy(), hf)
    assert np.array_equal(dmask.cpu().numpy(), hm)
    np.testing.assert_allclose(da.cpu().numpy(), ha, rtol=1e-13, atol=1e-18)


def test_device_mesh_level8_counts_and_area(gpu_ctx):
    import math

    import torch

    from lpm_gb300 import core

    vx, fx, fa, fm = core.build_mesh_device(gpu_ctx, core.MESH_ICOS_TRI, 8)
    torch.cuda.synchronize()
    leaf = fm == 0
    assert int(leaf.sum()) == 1310720 and vx.shape[0] == 655362
    assert float(fa[leaf].sum()) == pytest.approx(4 * math.pi, rel=1e-12)
    r = torch.linalg.norm(vx, dim=1)
    assert float((r - 1).abs().max()) < 1e-15
