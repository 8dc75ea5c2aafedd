"""Mesh generator: LDU ordering, closed cells, the 1M-cell contraction sizes."""
import numpy as np

from rheotool_gb300.mesh import cavity_mesh, channel_mesh, contraction_mesh, graded_nodes


def test_graded_nodes():
    x = graded_nodes(0.0, 1.0, 10, 4.0)
    d = np.diff(x)
    assert abs(d[-1] / d[0] - 4.0) < 1e-12 and abs(x[-1] - 1.0) < 1e-15


def test_cavity_addressing():
    m = cavity_mesh(8)
    m.check()
    assert m.nCells == 64 and m.nFaces == 2 * 7 * 8 and m.nBFaces == 32
    assert [p.name for p in m.patches] == ["movingLid", "fixedWalls"]
    assert np.all(m.Cf[:, 2] == 0.0)


def test_contraction_million_cells():
    m = contraction_mesh()
    assert m.nCells == 1_000_000
    m.check()
    # volume = upstream 20x8x2 + downstream 20x2x2
    assert abs(m.V.sum() - (20 * 8 * 2 + 20 * 2 * 2)) < 1e-8
    nb = np.bincount(m.bPatch)
    assert nb[0] == 100 * 50 and nb[1] == 50 * 50


def test_contraction_small_closed():
    m = contraction_mesh(6, 5, 4, 2, 3, 2.0, 2.0)
    m.check()
    assert np.all(m.w > 0) and np.all(m.w < 1)
    # every cell is bounded by 6 faces (internal + boundary)
    cnt = np.bincount(m.owner, minlength=m.nCells) + np.bincount(m.neighbour, minlength=m.nCells) \
        + np.bincount(m.bCell, minlength=m.nCells)
    assert np.all(cnt == 6)


def test_channel_2d():
    m = channel_mesh(5, 4, 1, two_d=True)
    m.check()
    assert list(m.solveDir) == [1, 1, 0]
