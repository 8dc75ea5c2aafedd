"""Rectilinear hex meshes in OpenFOAM LDU (face-addressed) form.

The meshes are what OpenFOAM's ``blockMesh`` builds for axis-aligned blocks
(``system/blockMeshDict`` with ``simpleGrading``), restated in numpy:

* cells are the active cells of an ``nx x ny x nz`` box grid, numbered
  lexicographically (i fastest, then j, then k); inactive cells make holes,
  which is how the 4:1 contraction (two blocks of different height) is built;
* internal faces are in upper-triangular order: sorted by owner, then by
  neighbour, with ``owner < neighbour`` (the order ``lduAddressing`` expects,
  ``eigenSolver.C:581-620`` in rheoTool reads the matrix with it);
* boundary faces are grouped patch by patch; ``empty`` patches (the front and
  back of a 2-D case) carry no faces at all, as in OpenFOAM;
* geometry follows ``surfaceInterpolation``: linear weights
  ``w = |Sf.(C_N - Cf)| / (|Sf.(Cf - C_P)| + |Sf.(C_N - Cf)|)`` and
  ``deltaCoeffs = 1/|C_N - C_P|``; boundary faces have ``w = 1`` and
  ``deltaCoeffs = 1/|Cf - C_P|`` (the faces are orthogonal, so the normal and
  the full distance agree).

Arrays are kept in OpenFOAM's own layout (AoS ``(n, 3)`` vectors) so that the
same object feeds both the C-ABI library and the FP64 CPU oracle.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

# direction codes for the six faces of a hex cell
XM, XP, YM, YP, ZM, ZP = range(6)
_DIRS = [(-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)]


def graded_nodes(x0: float, x1: float, n: int, ratio: float = 1.0) -> np.ndarray:
    """Node coordinates of ``n`` cells on [x0, x1] with blockMesh
    ``simpleGrading`` expansion ``ratio`` = last cell size / first cell size."""
    if n < 1:
        raise ValueError("need at least one cell")
    if ratio == 1.0 or n == 1:
        d = np.full(n, 1.0)
    else:
        q = ratio ** (1.0 / (n - 1))
        d = q ** np.arange(n, dtype=np.float64)
    s = np.concatenate([[0.0], np.cumsum(d)])
    s /= s[-1]
    x = x0 + (x1 - x0) * s
    x[0], x[-1] = x0, x1
    return x


def two_sided_nodes(x0: float, x1: float, n: int, ratio: float) -> np.ndarray:
    """Nodes clustered towards both ends (two blocks of n/2 cells, the second
    one with the inverse grading), the usual wall-refined channel spacing."""
    n1 = n // 2
    n2 = n - n1
    xm = 0.5 * (x0 + x1)
    a = graded_nodes(x0, xm, n1, ratio)
    b = graded_nodes(xm, x1, n2, 1.0 / ratio)
    return np.concatenate([a, b[1:]])


@dataclass
class Patch:
    name: str
    start: int
    size: int


@dataclass
class Mesh:
    nCells: int
    owner: np.ndarray
    neighbour: np.ndarray
    Sf: np.ndarray
    magSf: np.ndarray
    Cf: np.ndarray
    w: np.ndarray
    deltaCoeffs: np.ndarray
    C: np.ndarray
    V: np.ndarray
    bCell: np.ndarray
    bSf: np.ndarray
    bmagSf: np.ndarray
    bCf: np.ndarray
    bDelta: np.ndarray
    bPatch: np.ndarray
    patches: List[Patch]
    solveDir: np.ndarray            # (3,) int32, 0 where the direction is empty
    shape: Tuple[int, int, int]     # (nx, ny, nz) of the bounding grid
    cellIJK: np.ndarray             # (nCells, 3) int32 grid position
    name: str = "mesh"
    # cyclic (periodic) face pairs, stored as internal faces: C_N - C_P per
    # face with the neighbour translated by the period (None: C[N] - C[P]),
    # and a flag per face (None: no coupled faces)
    delta: Optional[np.ndarray] = None      # (nFaces, 3)
    coupled: Optional[np.ndarray] = None    # (nFaces,) int32

    @property
    def nFaces(self) -> int:
        return int(self.owner.shape[0])

    @property
    def nBFaces(self) -> int:
        return int(self.bCell.shape[0])

    def patch(self, name: str) -> Patch:
        for p in self.patches:
            if p.name == name:
                return p
        raise KeyError(name)

    def patch_id(self, name: str) -> int:
        for i, p in enumerate(self.patches):
            if p.name == name:
                return i
        raise KeyError(name)

    def check(self) -> None:
        """Cheap consistency checks of the LDU addressing."""
        o, n = self.owner, self.neighbour
        assert np.all(o < n), "owner must be below neighbour"
        key = o.astype(np.int64) * self.nCells + n
        assert np.all(np.diff(key) > 0), "faces must be in upper-triangular order"
        # closed cells: sum of outward area vectors is zero
        s = np.zeros((self.nCells, 3))
        np.add.at(s, o, self.Sf)
        np.add.at(s, n, -self.Sf)
        np.add.at(s, self.bCell, self.bSf)
        if self.solveDir.min() == 1:
            scale = np.abs(self.Sf).max()
            assert np.abs(s).max() < 1e-9 * scale, "cells are not closed"


def structured_mesh(
    xs: np.ndarray,
    ys: np.ndarray,
    zs: np.ndarray,
    patch_of: Callable[[int, np.ndarray, np.ndarray, np.ndarray, np.ndarray], np.ndarray],
    patch_names: Sequence[str],
    active: Optional[np.ndarray] = None,
    empty_z: bool = False,
    name: str = "mesh",
    periodic: Sequence[bool] = (False, False, False),
) -> Mesh:
    """Build an LDU mesh from node coordinates and an active-cell mask.

    ``patch_of(direction, i, j, k, Cf)`` returns, for the boundary faces of the
    given direction at cells (i, j, k) with face centres Cf (m, 3), an integer
    array of indices into ``patch_names``, or -1 for an empty face.

    ``periodic[d]`` joins the two ends of direction d (x, y, z) by a cyclic
    patch pair: each pair of end cells shares one internal face, owned by the
    lower-numbered cell (the one at index 0) and placed at that cell's end of
    the box, with the neighbour centre translated by the period for the
    weights, the deltaCoeffs and the face delta vector.  Such faces are
    flagged in ``Mesh.coupled`` (they act in the matrix but, like OpenFOAM's
    cyclic lduInterfaces, not in the DIC/DILU preconditioners).  A periodic
    direction needs at least 3 cells and no holes at its ends.
    """
    xs, ys, zs = (np.asarray(a, dtype=np.float64) for a in (xs, ys, zs))
    nx, ny, nz = len(xs) - 1, len(ys) - 1, len(zs) - 1
    if active is None:
        active = np.ones((nz, ny, nx), dtype=bool)
    assert active.shape == (nz, ny, nx)
    xc, yc, zc = 0.5 * (xs[:-1] + xs[1:]), 0.5 * (ys[:-1] + ys[1:]), 0.5 * (zs[:-1] + zs[1:])
    dx, dy, dz = np.diff(xs), np.diff(ys), np.diff(zs)

    idx = -np.ones((nz, ny, nx), dtype=np.int64)
    kk, jj, ii = np.nonzero(active)          # lexicographic with i fastest
    N = kk.size
    idx[kk, jj, ii] = np.arange(N)
    C = np.stack([xc[ii], yc[jj], zc[kk]], axis=1)
    V = dx[ii] * dy[jj] * dz[kk]

    periodic = tuple(bool(p) for p in periodic)
    dims = (nx, ny, nz)
    for a, per in enumerate(periodic):
        if not per:
            continue
        if dims[a] < 3 or (a == 2 and empty_z):
            raise ValueError("a periodic direction needs at least 3 cells (and cannot be empty)")
        ends = np.take(active, [0, dims[a] - 1], axis=2 - a)
        if not ends.all():
            raise ValueError("a periodic direction cannot have holes at its ends")
    period = np.array([xs[-1] - xs[0], ys[-1] - ys[0], zs[-1] - zs[0]])

    # ---- internal faces --------------------------------------------------
    own_l, nei_l, Sf_l, Cf_l, sh_l, cp_l = [], [], [], [], [], []
    for d, (di, dj, dk) in ((XP, _DIRS[XP]), (YP, _DIRS[YP]), (ZP, _DIRS[ZP])):
        i2, j2, k2 = ii + di, jj + dj, kk + dk
        inside = (i2 < nx) & (j2 < ny) & (k2 < nz)
        nb = np.full(N, -1, dtype=np.int64)
        nb[inside] = idx[k2[inside], j2[inside], i2[inside]]
        m = nb >= 0
        if d == ZP and empty_z:
            m &= False
        c = np.nonzero(m)[0]
        own_l.append(c)
        nei_l.append(nb[m])
        S = np.zeros((c.size, 3))
        F = np.zeros((c.size, 3))
        if d == XP:
            S[:, 0] = dy[jj[c]] * dz[kk[c]]
            F[:] = np.stack([xs[ii[c] + 1], yc[jj[c]], zc[kk[c]]], axis=1)
        elif d == YP:
            S[:, 1] = dx[ii[c]] * dz[kk[c]]
            F[:] = np.stack([xc[ii[c]], ys[jj[c] + 1], zc[kk[c]]], axis=1)
        else:
            S[:, 2] = dx[ii[c]] * dy[jj[c]]
            F[:] = np.stack([xc[ii[c]], yc[jj[c]], zs[kk[c] + 1]], axis=1)
        Sf_l.append(S)
        Cf_l.append(F)
        sh_l.append(np.zeros((c.size, 3)))
        cp_l.append(np.zeros(c.size, np.int32))
        a = (XP, YP, ZP).index(d)
        if periodic[a]:
            # the cyclic pair: owner at index 0, neighbour at the far end
            pos = (ii, jj, kk)[a]
            lo = np.nonzero(pos == 0)[0]
            far = [ii[lo], jj[lo], kk[lo]]
            far[a] = np.full(lo.size, dims[a] - 1)
            nbw = idx[far[2], far[1], far[0]]
            S = np.zeros((lo.size, 3))
            F = np.stack([xc[ii[lo]], yc[jj[lo]], zc[kk[lo]]], axis=1)
            area = (dy[jj[lo]] * dz[kk[lo]], dx[ii[lo]] * dz[kk[lo]], dx[ii[lo]] * dy[jj[lo]])[a]
            S[:, a] = -area                        # outward from the owner, towards -axis
            F[:, a] = (xs, ys, zs)[a][0]
            shift = np.zeros((lo.size, 3))
            shift[:, a] = -period[a]               # the neighbour's image next to the owner
            own_l.append(lo)
            nei_l.append(nbw)
            Sf_l.append(S)
            Cf_l.append(F)
            sh_l.append(shift)
            cp_l.append(np.ones(lo.size, np.int32))
    owner = np.concatenate(own_l)
    neighbour = np.concatenate(nei_l)
    Sf = np.concatenate(Sf_l)
    Cf = np.concatenate(Cf_l)
    shift = np.concatenate(sh_l)
    coupled = np.concatenate(cp_l)
    order = np.lexsort((neighbour, owner))
    owner, neighbour, Sf, Cf = owner[order], neighbour[order], Sf[order], Cf[order]
    shift, coupled = shift[order], coupled[order]
    CN = C[neighbour] + shift
    magSf = np.sqrt((Sf * Sf).sum(1))
    sfdOwn = np.abs((Sf * (Cf - C[owner])).sum(1))
    sfdNei = np.abs((Sf * (CN - Cf)).sum(1))
    w = sfdNei / (sfdOwn + sfdNei)
    dvec = CN - C[owner]
    deltaCoeffs = 1.0 / np.sqrt((dvec * dvec).sum(1))
    anyPeriodic = any(periodic)

    # ---- boundary faces ------------------------------------------------------
    b_cell, b_dir, b_patch, b_Sf, b_Cf = [], [], [], [], []
    for d in range(6):
        di, dj, dk = _DIRS[d]
        i2, j2, k2 = ii + di, jj + dj, kk + dk
        out = (i2 < 0) | (i2 >= nx) | (j2 < 0) | (j2 >= ny) | (k2 < 0) | (k2 >= nz)
        nb = np.full(N, -1, dtype=np.int64)
        ins = ~out
        nb[ins] = idx[k2[ins], j2[ins], i2[ins]]
        c = np.nonzero(nb < 0)[0]
        if periodic[d // 2]:
            continue          # the ends of a periodic direction are joined
        if c.size == 0:
            continue
        S = np.zeros((c.size, 3))
        F = np.stack([xc[ii[c]], yc[jj[c]], zc[kk[c]]], axis=1)
        if d in (XM, XP):
            S[:, 0] = (1.0 if d == XP else -1.0) * dy[jj[c]] * dz[kk[c]]
            F[:, 0] = xs[ii[c] + (1 if d == XP else 0)]
        elif d in (YM, YP):
            S[:, 1] = (1.0 if d == YP else -1.0) * dx[ii[c]] * dz[kk[c]]
            F[:, 1] = ys[jj[c] + (1 if d == YP else 0)]
        else:
            S[:, 2] = (1.0 if d == ZP else -1.0) * dx[ii[c]] * dy[jj[c]]
            F[:, 2] = zs[kk[c] + (1 if d == ZP else 0)]
        pid = np.asarray(patch_of(d, ii[c], jj[c], kk[c], F), dtype=np.int64)
        if empty_z and d in (ZM, ZP):
            pid[:] = -1
        keep = pid >= 0
        b_cell.append(c[keep])
        b_dir.append(np.full(int(keep.sum()), d))
        b_patch.append(pid[keep])
        b_Sf.append(S[keep])
        b_Cf.append(F[keep])
    bCell = np.concatenate(b_cell) if b_cell else np.zeros(0, np.int64)
    bDir = np.concatenate(b_dir) if b_dir else np.zeros(0, np.int64)
    bPatch = np.concatenate(b_patch) if b_patch else np.zeros(0, np.int64)
    bSf = np.concatenate(b_Sf) if b_Sf else np.zeros((0, 3))
    bCf = np.concatenate(b_Cf) if b_Cf else np.zeros((0, 3))
    order = np.lexsort((bDir, bCell, bPatch))
    bCell, bPatch, bSf, bCf = bCell[order], bPatch[order], bSf[order], bCf[order]
    bmagSf = np.sqrt((bSf * bSf).sum(1))
    dv = bCf - C[bCell]
    bDelta = 1.0 / np.sqrt((dv * dv).sum(1))
    patches = []
    for p, nm in enumerate(patch_names):
        sel = np.nonzero(bPatch == p)[0]
        start = int(sel[0]) if sel.size else int(np.searchsorted(bPatch, p))
        patches.append(Patch(nm, start, int(sel.size)))

    solveDir = np.array([1, 1, 0 if empty_z else 1], dtype=np.int32)
    m = Mesh(
        nCells=N,
        owner=owner.astype(np.int32), neighbour=neighbour.astype(np.int32),
        Sf=np.ascontiguousarray(Sf), magSf=magSf, Cf=np.ascontiguousarray(Cf), w=w,
        deltaCoeffs=deltaCoeffs, C=np.ascontiguousarray(C), V=V,
        bCell=bCell.astype(np.int32), bSf=np.ascontiguousarray(bSf), bmagSf=bmagSf,
        bCf=np.ascontiguousarray(bCf), bDelta=bDelta, bPatch=bPatch.astype(np.int32),
        patches=patches, solveDir=solveDir, shape=(nx, ny, nz),
        cellIJK=np.stack([ii, jj, kk], axis=1).astype(np.int32), name=name,
        delta=np.ascontiguousarray(dvec) if anyPeriodic else None,
        coupled=coupled if anyPeriodic else None,
    )
    return m


# ---------------------------------------------------------------------------
# The meshes of the workloads
# ---------------------------------------------------------------------------

def cavity_mesh(n: int = 64, ny: Optional[int] = None) -> Mesh:
    """Unit lid-driven cavity [0,1]^2 x [-0.5,0.5], ``n x n x 1`` uniform hex
    cells, patches ``movingLid`` (y=1), ``fixedWalls`` and an empty
    ``frontAndBack`` (the rheoTool ``Cavity`` tutorial layout)."""
    ny = n if ny is None else ny
    xs = graded_nodes(0.0, 1.0, n)
    ys = graded_nodes(0.0, 1.0, ny)
    zs = np.array([-0.5, 0.5])

    def patch_of(d, i, j, k, Cf):
        if d == YP:
            return np.zeros(i.size, np.int64)
        if d in (ZM, ZP):
            return -np.ones(i.size, np.int64)
        return np.ones(i.size, np.int64)

    return structured_mesh(xs, ys, zs, patch_of, ["movingLid", "fixedWalls"],
                           empty_z=True, name=f"cavity{n}x{ny}")


def contraction_mesh(nx_up: int = 134, nx_down: int = 132, ny_in: int = 50,
                     ny_out: int = 25, nz: int = 50, L_up: float = 20.0,
                     L_down: float = 20.0, depth: float = 2.0,
                     name: Optional[str] = None, two_d: bool = False) -> Mesh:
    """3-D planar 4:1 contraction: upstream channel y in [-4, 4], downstream
    y in [-1, 1] (H = 1), depth ``depth`` in z, the contraction plane at x = 0.

    The bounding grid is (nx_up + nx_down) x (ny_in + 2 ny_out) x nz; the
    cells with x > 0 and |y| > 1 are holes.  Spacing is refined towards the
    contraction plane in x, towards the re-entrant corners y = +-1 and towards
    the z walls.  Patches: ``inlet`` (x = -L_up), ``outlet`` (x = L_down) and
    ``walls`` (everything else).  The default sizes give exactly 1,000,000
    cells: 50 * (134 * 100 + 132 * 50).  ``two_d``: one cell thick with empty
    front and back (the planar 2-D contraction; nz is then 1).
    """
    if two_d:
        nz = 1
    xs_up = graded_nodes(-L_up, 0.0, nx_up, 1.0 / 20.0)
    xs_dn = graded_nodes(0.0, L_down, nx_down, 20.0)
    xs = np.concatenate([xs_up, xs_dn[1:]])
    y_lo = graded_nodes(-4.0, -1.0, ny_out, 1.0 / 8.0)
    y_mid = two_sided_nodes(-1.0, 1.0, ny_in, 4.0)
    y_hi = graded_nodes(1.0, 4.0, ny_out, 8.0)
    ys = np.concatenate([y_lo, y_mid[1:], y_hi[1:]])
    zs = np.array([0.0, depth]) if two_d else two_sided_nodes(0.0, depth, nz, 4.0)
    nx, ny = len(xs) - 1, len(ys) - 1
    active = np.ones((nz, ny, nx), dtype=bool)
    # holes: downstream (i >= nx_up) outside the narrow channel
    active[:, :ny_out, nx_up:] = False
    active[:, ny_out + ny_in:, nx_up:] = False

    def patch_of(d, i, j, k, Cf):
        p = np.full(i.size, 2, np.int64)
        if d == XM:
            p[i == 0] = 0
        if d == XP:
            p[i == nx - 1] = 1
        return p

    N = nz * (nx_up * ny + nx_down * ny_in)
    return structured_mesh(xs, ys, zs, patch_of, ["inlet", "outlet", "walls"],
                           active=active, empty_z=two_d, name=name or f"contraction{N}")


def channel_mesh(nx: int = 20, ny: int = 16, nz: int = 4, L: float = 4.0,
                 H: float = 1.0, depth: float = 1.0, two_d: bool = False) -> Mesh:
    """Straight channel with ``inlet``/``outlet``/``walls`` (walls at y = 0, H
    and, in 3-D, at z = 0, depth); used for Poiseuille checks."""
    xs = graded_nodes(0.0, L, nx)
    ys = graded_nodes(0.0, H, ny)
    zs = graded_nodes(0.0, depth, nz) if not two_d else np.array([0.0, depth])

    def patch_of(d, i, j, k, Cf):
        p = np.full(i.size, 2, np.int64)
        if d == XM:
            p[:] = 0
        if d == XP:
            p[:] = 1
        return p

    return structured_mesh(xs, ys, zs, patch_of, ["inlet", "outlet", "walls"],
                           empty_z=two_d, name=f"channel{nx}x{ny}x{nz}")


def periodic_channel_mesh(nx: int = 400, ny: int = 100, nz: int = 100, L: float = 8.0,
                          H: float = 1.0, depth: float = 4.0, wall_ratio: float = 4.0) -> Mesh:
    """3-D channel, periodic (cyclic) in the streamwise x and spanwise z
    directions, walls at y = -H and y = +H (patch ``walls``, the only patch).
    The wall-normal spacing is refined towards both walls (``wall_ratio`` =
    centre cell height / wall cell height); x and z are uniform.  The
    defaults give 4,000,000 cells."""
    xs = graded_nodes(0.0, L, nx)
    ys = two_sided_nodes(-H, H, ny, wall_ratio) if wall_ratio != 1.0 else graded_nodes(-H, H, ny)
    zs = graded_nodes(0.0, depth, nz)

    def patch_of(d, i, j, k, Cf):
        return np.zeros(i.size, np.int64)

    return structured_mesh(xs, ys, zs, patch_of, ["walls"], periodic=(True, False, True),
                           name=f"periodicChannel{nx}x{ny}x{nz}")
