"""The batched form's disjoint union of meshes, on the CPU: a valid LDU mesh
(upper-triangular face order kept, cells closed), case ranges that cover
cells, faces and boundary faces, per-case patches renamed, geometry carried
over unchanged, and mixed empty directions refused."""
import numpy as np
import pytest

from rheotool_gb300.batch import union_mesh
from rheotool_gb300.mesh import cavity_mesh, channel_mesh


def test_union_of_cavities():
    ms = [cavity_mesh(n) for n in (5, 8, 3)]
    u, cs, fs, bs = union_mesh(ms)
    u.check()
    assert list(cs) == [0, 25, 89, 98]
    assert fs[-1] == u.nFaces == sum(m.nFaces for m in ms)
    assert bs[-1] == u.nBFaces == sum(m.nBFaces for m in ms)
    for i, m in enumerate(ms):
        o = u.owner[fs[i]:fs[i + 1]] - cs[i]
        n = u.neighbour[fs[i]:fs[i + 1]] - cs[i]
        assert np.array_equal(o, m.owner) and np.array_equal(n, m.neighbour)
        assert np.array_equal(u.V[cs[i]:cs[i + 1]], m.V)
        assert np.array_equal(u.bCell[bs[i]:bs[i + 1]] - cs[i], m.bCell)
        names = [p.name for p in u.patches if p.name.startswith(f"{i}:")]
        assert names == [f"{i}:{p.name}" for p in m.patches]
        for p in m.patches:
            q = next(x for x in u.patches if x.name == f"{i}:{p.name}")
            assert q.start == bs[i] + p.start and q.size == p.size
    # faces never leave their case
    case_of = np.repeat(np.arange(len(ms)), np.diff(cs))
    assert np.array_equal(case_of[u.owner], case_of[u.neighbour])


def test_union_refuses_mixed_empty_directions():
    with pytest.raises(ValueError, match="empty directions"):
        union_mesh([cavity_mesh(4), channel_mesh(nx=4, ny=3, nz=2)])
