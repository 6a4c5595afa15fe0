"""Host-side octree and target blocks of the far field (no GPU): leaves hold
at most leaf_max points, the source order is a permutation, children tile
their parent's range, every target is in exactly one block of <= 128."""
import numpy as np
import pytest


@pytest.mark.parametrize("level,leaf", [(4, 64), (5, 64), (5, 16)])
def test_octree_structure(level, leaf):
    from lpm_gb300 import core
    from lpm_gb300.farfield import octree_stats

    vx, fx, fa, fm = core.build_mesh(core.MESH_ICOS_TRI, level, 1.0)
    src = fx[fm == 0]
    tgt = np.concatenate([vx, src])
    st = octree_stats(src, tgt, leaf)
    assert st["errors"] == 0
    assert st["max_leaf"] <= leaf
    assert st["sources_in_leaves"] == src.shape[0]
    assert st["targets_covered"] == tgt.shape[0]
    assert st["blocks"] <= 3 * (tgt.shape[0] // 128 + 1)  # blocks stay well filled
    assert st["min_block_fill"] >= 1


def test_octree_duplicate_points_terminate():
    """Coincident points cannot be separated: the split stops at the deepest
    level and the leaf keeps them all."""
    from lpm_gb300.farfield import octree_stats

    src = np.repeat(np.array([[0.0, 0.0, 1.0]]), 100, axis=0)
    src = np.concatenate([src, np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])])
    st = octree_stats(src, src, 64)
    assert st["errors"] == 0 and st["max_leaf"] == 100 and st["max_level"] == 21


def test_octree_rejects_bad_arguments():
    from lpm_gb300.core import LpmError
    from lpm_gb300.farfield import octree_stats

    with pytest.raises(LpmError):
        octree_stats(np.zeros((0, 3)), np.zeros((0, 3)))
    with pytest.raises(LpmError):
        octree_stats(np.zeros((4, 3)), np.zeros((1, 3)), leaf_max=65)
