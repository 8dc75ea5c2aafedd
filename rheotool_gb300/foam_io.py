"""OpenFOAM case I/O: the ``constant/polyMesh`` reader and ASCII field files.

The reader turns an OpenFOAM polyMesh (``points``, ``faces``, ``owner``,
``neighbour``, ``boundary``; ASCII or binary format, plain or ``.gz``) into
the LDU ``Mesh`` the library and the oracle take:

* geometry as OpenFOAM's ``primitiveMesh`` defines it: a face's centre and
  area vector from the triangles joining each edge to the mean of its points
  (area-weighted triangle centroids, half the sum of the triangle normals);
  a cell's centre and volume from the pyramids joining each face to the mean
  of the cell's face centres (volume-weighted pyramid centroids at 3/4 of the
  way from apex to base);
* ``surfaceInterpolation`` weights ``w = |Sf.(C_N - Cf)| / (|Sf.(Cf - C_P)| +
  |Sf.(C_N - Cf)|)`` and ``deltaCoeffs = 1/|C_N - C_P|``; boundary faces
  ``deltaCoeffs = 1/|Cf - C_P|``;
* ``empty`` patches carry no faces and mark their normal direction as not
  solved (``solutionD``);
* each ``cyclic`` patch pair becomes coupled internal faces (owner the lower
  cell, area vector outward from it, neighbour centre translated by the
  separation of the two patch faces), in upper-triangular order with the
  other internal faces.  ``Mesh.foamFace`` records, for every LDU face, the
  OpenFOAM face it came from (for a cyclic pair, the face on the owner's
  patch) and ``Mesh.foamPartner`` the pair's other face, which the field
  writer uses to put ``phi`` back on both cyclic patches.

The field writer emits ``volScalarField`` / ``volVectorField`` /
``volSymmTensorField`` / ``volTensorField`` / ``surfaceScalarField`` files in
OpenFOAM's ASCII format with ``writePrecision`` significant digits (the
reference cases write 12), ``nonuniform`` internal fields and per-patch
boundary values.  ``read_field`` reads back ``uniform`` and ``nonuniform``
internal fields and boundary ``value`` entries.
"""
from __future__ import annotations

import gzip
import os
import re
from typing import Dict, List, Optional, Tuple

import numpy as np

from .mesh import Mesh, Patch

# ---------------------------------------------------------------------------
# tokenising
# ---------------------------------------------------------------------------
_COMMENT = re.compile(r"//[^\n]*|/\*.*?\*/", re.S)


def _read_text(path: str) -> str:
    for p in (path, path + ".gz"):
        if os.path.exists(p):
            if p.endswith(".gz"):
                with gzip.open(p, "rt") as f:
                    return f.read()
            with open(p) as f:
                return f.read()
    raise FileNotFoundError(path)


def _strip(text: str) -> str:
    return _COMMENT.sub(" ", text)


def _body(text: str) -> str:
    """The file without comments and without its FoamFile header."""
    t = _strip(text)
    m = re.search(r"\bFoamFile\s*\{", t)
    if m:
        depth, i = 1, m.end()
        while depth and i < len(t):
            if t[i] == "{":
                depth += 1
            elif t[i] == "}":
                depth -= 1
            i += 1
        t = t[i:]
    return t


def _header(text: str) -> Dict[str, str]:
    t = _strip(text)
    m = re.search(r"\bFoamFile\s*\{(.*?)\}", t, re.S)
    out = {}
    if m:
        for k, v in re.findall(r"(\w+)\s+([^;]*);", m.group(1)):
            out[k] = v.strip().strip('"')
    return out


def _list_span(t: str, start: int = 0) -> Tuple[int, int, int]:
    """(count, index after '(', index of the matching ')') of the first
    ``N ( ... )`` list at or after ``start``."""
    m = re.compile(r"(\d+)\s*\(").search(t, start)
    if not m:
        raise ValueError("no list found")
    n = int(m.group(1))
    depth, i = 1, m.end()
    while depth:
        c = t[i]
        if c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
        i += 1
    return n, m.end(), i - 1


def _numbers(s: str) -> np.ndarray:
    s = s.replace("(", " ").replace(")", " ")
    return np.array(s.split(), dtype=np.float64) if s.strip() else np.zeros(0)


def _read_bytes(path: str) -> bytes:
    for p in (path, path + ".gz"):
        if os.path.exists(p):
            if p.endswith(".gz"):
                with gzip.open(p, "rb") as f:
                    return f.read()
            with open(p, "rb") as f:
                return f.read()
    raise FileNotFoundError(path)


def _binary_header(raw: bytes) -> Optional[Dict[str, str]]:
    """The FoamFile header of a binary-format file (None for ASCII)."""
    head = raw[:4096].decode("latin-1")
    h = _header(head)
    return h if h.get("format", "ascii") == "binary" else None


def _binary_lists(raw: bytes, dtypes: List[np.dtype], widths: List[int]) -> List[np.ndarray]:
    """The raw lists ``N ( <N x width items of dtype> )`` that follow the
    header of a binary-format file, in order."""
    pos = raw.index(b"}", raw.index(b"FoamFile")) + 1
    out = []
    for dt, wdt in zip(dtypes, widths):
        m = re.compile(rb"(\d+)\s*\(").search(raw, pos)
        if not m:
            raise ValueError("binary list not found")
        n = int(m.group(1))
        nbytes = n * wdt * dt.itemsize
        a = m.end()
        out.append(np.frombuffer(raw[a:a + nbytes], dtype=dt).reshape(n, wdt) if wdt > 1
                   else np.frombuffer(raw[a:a + nbytes], dtype=dt).copy())
        pos = a + nbytes + 1      # past ')'
    return out


def _label_dtype(h: Dict[str, str]) -> np.dtype:
    return np.dtype(np.int64) if "label=64" in h.get("arch", "") else np.dtype(np.int32)


def _scalar_dtype(h: Dict[str, str]) -> np.dtype:
    return np.dtype(np.float32) if "scalar=32" in h.get("arch", "") else np.dtype(np.float64)


def read_label_list(path: str) -> np.ndarray:
    raw = _read_bytes(path)
    hb = _binary_header(raw)
    if hb is not None:
        return _binary_lists(raw, [_label_dtype(hb)], [1])[0].astype(np.int64)
    t = _body(raw.decode("latin-1"))
    n, a, b = _list_span(t)
    v = np.array(t[a:b].split(), dtype=np.int64)
    if v.size != n:
        raise ValueError(f"{path}: {v.size} labels, header says {n}")
    return v


def read_vector_list(path: str) -> np.ndarray:
    raw = _read_bytes(path)
    hb = _binary_header(raw)
    if hb is not None:
        return _binary_lists(raw, [_scalar_dtype(hb)], [3])[0].astype(np.float64)
    t = _body(raw.decode("latin-1"))
    n, a, b = _list_span(t)
    v = _numbers(t[a:b]).reshape(-1, 3)
    if v.shape[0] != n:
        raise ValueError(f"{path}: {v.shape[0]} vectors, header says {n}")
    return v


def read_faces(path: str) -> List[np.ndarray]:
    """faceList: ``N ( k(a b c ...) ... )``; also faceCompactList (offsets
    then labels), which is how binary files store the faces."""
    raw = _read_bytes(path)
    hb = _binary_header(raw)
    if hb is not None:
        ld = _label_dtype(hb)
        offs, lab = _binary_lists(raw, [ld, ld], [1, 1])
        offs, lab = offs.astype(np.int64), lab.astype(np.int64)
        return [lab[offs[i]:offs[i + 1]] for i in range(len(offs) - 1)]
    text = raw.decode("latin-1")
    t = _body(text)
    if "faceCompactList" in _header(text).get("class", ""):
        n1, a1, b1 = _list_span(t)
        offs = np.array(t[a1:b1].split(), dtype=np.int64)
        n2, a2, b2 = _list_span(t, b1 + 1)
        lab = np.array(t[a2:b2].split(), dtype=np.int64)
        return [lab[offs[i]:offs[i + 1]] for i in range(len(offs) - 1)]
    n, a, b = _list_span(t)
    faces = [np.array(m.group(2).split(), dtype=np.int64)
             for m in re.finditer(r"(\d+)\s*\(([^()]*)\)", t[a:b])]
    if len(faces) != n:
        raise ValueError(f"{path}: {len(faces)} faces, header says {n}")
    return faces


def read_boundary(path: str) -> List[Dict[str, str]]:
    t = _body(_read_text(path))
    n, a, b = _list_span(t)
    out = []
    for m in re.finditer(r"(\w+)\s*\{([^{}]*)\}", t[a:b]):
        d = {"name": m.group(1)}
        for k, v in re.findall(r"(\w+)\s+([^;]*);", m.group(2)):
            d[k] = v.strip()
        out.append(d)
    if len(out) != n:
        raise ValueError(f"{path}: {len(out)} patches, header says {n}")
    return out


# ---------------------------------------------------------------------------
# geometry (primitiveMesh's face and cell decompositions, restated)
# ---------------------------------------------------------------------------
def face_geometry(points: np.ndarray, faces: List[np.ndarray]) -> Tuple[np.ndarray, np.ndarray]:
    """Face centres and area vectors."""
    nF = len(faces)
    Cf = np.zeros((nF, 3))
    Sf = np.zeros((nF, 3))
    sizes = np.array([len(f) for f in faces])
    for k in np.unique(sizes):
        idx = np.nonzero(sizes == k)[0]
        P = points[np.stack([faces[i] for i in idx])]            # (m, k, 3)
        if k == 3:
            Cf[idx] = P.mean(1)
            Sf[idx] = 0.5 * np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0])
            continue
        c0 = P.mean(1)                                           # centre estimate
        Pn = np.roll(P, -1, axis=1)
        n = np.cross(Pn - P, c0[:, None, :] - P)                 # triangle normals (x2)
        c = P + Pn + c0[:, None, :]                              # triangle centroids (x3)
        a = np.linalg.norm(n, axis=2)
        sumA = a.sum(1)
        sumAc = (a[:, :, None] * c).sum(1)
        ok = sumA > 1e-300
        Cf[idx] = np.where(ok[:, None], sumAc / (3.0 * np.where(ok, sumA, 1.0)[:, None]), c0)
        Sf[idx] = 0.5 * n.sum(1)
    return Cf, Sf


def cell_geometry(nCells: int, owner: np.ndarray, neighbour: np.ndarray, Cf: np.ndarray,
                  Sf: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """Cell centres and volumes (owner: every face; neighbour: internal faces)."""
    nI = neighbour.size
    cnt = np.bincount(owner, minlength=nCells) + np.bincount(neighbour, minlength=nCells)
    cEst = np.zeros((nCells, 3))
    np.add.at(cEst, owner, Cf)
    np.add.at(cEst, neighbour, Cf[:nI])
    cEst /= cnt[:, None]
    v_o = (Sf * (Cf - cEst[owner])).sum(1)                       # 3 x pyramid volume
    v_n = (Sf[:nI] * (cEst[neighbour] - Cf[:nI])).sum(1)
    c_o = 0.75 * Cf + 0.25 * cEst[owner]
    c_n = 0.75 * Cf[:nI] + 0.25 * cEst[neighbour]
    vol = np.zeros(nCells)
    ctr = np.zeros((nCells, 3))
    np.add.at(vol, owner, v_o)
    np.add.at(vol, neighbour, v_n)
    np.add.at(ctr, owner, v_o[:, None] * c_o)
    np.add.at(ctr, neighbour, v_n[:, None] * c_n)
    ok = np.abs(vol) > 1e-300
    C = np.where(ok[:, None], ctr / np.where(ok, vol, 1.0)[:, None], cEst)
    return C, vol / 3.0


def mesh_quality(mesh: Mesh) -> Dict[str, float]:
    """Maximum non-orthogonality (degrees between the face normal and C_N - C_P)
    and maximum face skewness (distance of the face centre from the line
    C_P C_N, over |C_N - C_P|) of the internal faces.  The library's
    laplacian and face gradients are the orthogonal ones, exact only when the
    non-orthogonality is zero."""
    if mesh.nFaces == 0:
        return {"nonOrthogonality": 0.0, "skewness": 0.0}
    d = mesh.delta if mesh.delta is not None else mesh.C[mesh.neighbour] - mesh.C[mesh.owner]
    n = mesh.Sf / mesh.magSf[:, None]
    dl = np.linalg.norm(d, axis=1)
    cosang = np.clip((n * d).sum(1) / dl, -1.0, 1.0)
    nonorth = float(np.degrees(np.arccos(cosang)).max())
    # face centre relative to the owner centre, its part off the line P-N
    r = mesh.Cf - mesh.C[mesh.owner]
    t = (r * d).sum(1) / (dl * dl)
    off = np.linalg.norm(r - t[:, None] * d, axis=1)
    return {"nonOrthogonality": nonorth, "skewness": float((off / dl).max())}


# ---------------------------------------------------------------------------
# polyMesh -> LDU mesh
# ---------------------------------------------------------------------------
def read_polymesh(case_dir: str, name: Optional[str] = None) -> Mesh:
    """Read ``case_dir/constant/polyMesh`` (or ``case_dir`` itself when it is
    the polyMesh directory) into an LDU ``Mesh``."""
    d = case_dir
    if not os.path.exists(os.path.join(d, "owner")) and not os.path.exists(os.path.join(d, "owner.gz")):
        d = os.path.join(case_dir, "constant", "polyMesh")
    points = read_vector_list(os.path.join(d, "points"))
    faces = read_faces(os.path.join(d, "faces"))
    own = read_label_list(os.path.join(d, "owner"))
    nei = read_label_list(os.path.join(d, "neighbour"))
    bnd = read_boundary(os.path.join(d, "boundary"))
    nFaces = len(faces)
    nI = nei.size
    nCells = int(own.max()) + 1 if own.size else 0
    if nI:
        nCells = max(nCells, int(nei.max()) + 1)
    Cf, Sf = face_geometry(points, faces)
    C, V = cell_geometry(nCells, own, nei, Cf, Sf)

    # ---- patches: empty dropped, cyclic pairs folded into internal faces
    byname = {p["name"]: p for p in bnd}
    solve = np.ones(3, np.int32)
    kept, cyc_faces, cyc_seen = [], [], set()
    for p in bnd:
        s, n = int(p["startFace"]), int(p["nFaces"])
        typ = p.get("type", "patch")
        if typ == "empty":
            if n:
                a = np.abs(Sf[s:s + n]).sum(0)
                solve[a > 1e-12 * a.max()] = 0
            continue
        if typ == "cyclic":
            other = p.get("neighbourPatch")
            if other is None or other not in byname:
                raise ValueError(f"cyclic patch {p['name']} has no neighbourPatch")
            if p["name"] in cyc_seen:
                continue
            q = byname[other]
            cyc_seen.update([p["name"], other])
            sq, nq = int(q["startFace"]), int(q["nFaces"])
            if nq != n:
                raise ValueError(f"cyclic pair {p['name']}/{other}: {n} and {nq} faces")
            cyc_faces.append((np.arange(s, s + n), np.arange(sq, sq + n)))
            continue
        kept.append((p["name"], s, n))

    # ---- internal faces, then the coupled cyclic faces
    o = own[:nI].copy()
    nb = nei.copy()
    iSf = Sf[:nI].copy()
    iCf = Cf[:nI].copy()
    shift = np.zeros((nI, 3))
    coupled = np.zeros(nI, np.int32)
    src = np.arange(nI)
    partner = np.full(nI, -1, dtype=np.int64)   # the other patch face of a cyclic pair
    for fa, fb in cyc_faces:
        ca, cb = own[fa], own[fb]
        sep = Cf[fa] - Cf[fb]                 # translation taking patch b onto patch a
        a_low = ca < cb
        lo = np.where(a_low, ca, cb)
        hi = np.where(a_low, cb, ca)
        sf = np.where(a_low[:, None], Sf[fa], Sf[fb])
        cf = np.where(a_low[:, None], Cf[fa], Cf[fb])
        # the neighbour's image next to the owner: across face a it is C_b + sep
        sh = np.where(a_low[:, None], sep, -sep)
        o = np.concatenate([o, lo])
        nb = np.concatenate([nb, hi])
        iSf = np.concatenate([iSf, sf])
        iCf = np.concatenate([iCf, cf])
        shift = np.concatenate([shift, sh])
        coupled = np.concatenate([coupled, np.ones(fa.size, np.int32)])
        src = np.concatenate([src, np.where(a_low, fa, fb)])
        partner = np.concatenate([partner, np.where(a_low, fb, fa)])
    if np.any(o == nb):
        raise ValueError("a cyclic face joins a cell to itself")
    order = np.lexsort((nb, o))
    o, nb, iSf, iCf, shift, coupled, src, partner = (x[order] for x in (o, nb, iSf, iCf, shift, coupled, src,
                                                                        partner))
    CN = C[nb] + shift
    magSf = np.linalg.norm(iSf, axis=1)
    sfdOwn = np.abs((iSf * (iCf - C[o])).sum(1))
    sfdNei = np.abs((iSf * (CN - iCf)).sum(1))
    w = sfdNei / (sfdOwn + sfdNei)
    dvec = CN - C[o]
    deltaCoeffs = 1.0 / np.linalg.norm(dvec, axis=1)

    # ---- boundary faces of the kept patches, patch by patch
    bsel, patches, start = [], [], 0
    for nm, s, n in kept:
        bsel.append(np.arange(s, s + n))
        patches.append(Patch(nm, start, n))
        start += n
    bidx = np.concatenate(bsel) if bsel else np.zeros(0, np.int64)
    bCell = own[bidx]
    bSf = Sf[bidx]
    bCf = Cf[bidx]
    bmagSf = np.linalg.norm(bSf, axis=1)
    dv = bCf - C[bCell]
    bDelta = 1.0 / np.linalg.norm(dv, axis=1)
    hasCyc = bool(cyc_faces)
    m = Mesh(
        nCells=nCells, owner=o.astype(np.int32), neighbour=nb.astype(np.int32),
        Sf=np.ascontiguousarray(iSf), magSf=magSf, Cf=np.ascontiguousarray(iCf), w=w,
        deltaCoeffs=deltaCoeffs, C=np.ascontiguousarray(C), V=V,
        bCell=bCell.astype(np.int32), bSf=np.ascontiguousarray(bSf), bmagSf=bmagSf,
        bCf=np.ascontiguousarray(bCf), bDelta=bDelta,
        bPatch=np.concatenate([np.full(n, i, np.int32) for i, (_, _, n) in enumerate(kept)])
        if kept else np.zeros(0, np.int32),
        patches=patches, solveDir=solve, shape=None, cellIJK=None,
        name=name or os.path.basename(os.path.abspath(case_dir)),
        delta=np.ascontiguousarray(dvec) if hasCyc else None,
        coupled=coupled if hasCyc else None,
    )
    m.foamFace = src.astype(np.int64)          # OpenFOAM face of each LDU face
    m.foamPartner = partner                    # for a cyclic pair, the face on the other patch
    m.foamBFace = bidx.astype(np.int64)        # OpenFOAM face of each boundary face
    m.foamPatches = bnd
    m.foamNFaces = nFaces
    return m


# ---------------------------------------------------------------------------
# structured meshes -> polyMesh files (blockMesh's point and face numbering)
# ---------------------------------------------------------------------------
def _fmt(x: float, prec: int) -> str:
    return f"{x:.{prec}g}"


def _header_text(cls: str, obj: str, location: str, note: Optional[str] = None) -> str:
    h = ("FoamFile\n{\n    version     2.0;\n    format      ascii;\n"
         f"    class       {cls};\n")
    if note:
        h += f'    note        "{note}";\n'
    h += f'    location    "{location}";\n    object      {obj};\n}}\n\n'
    return h


def write_structured_polymesh(out_dir: str, xs, ys, zs, patch_of, patch_names, patch_types=None,
                              empty_z: bool = False, periodic=(False, False, False), prec: int = 17) -> None:
    """Write the polyMesh of an axis-aligned box grid (all cells active),
    numbered as blockMesh numbers one block: points i fastest, cells i
    fastest, internal faces in upper-triangular order, boundary faces patch by
    patch.  ``patch_of(direction, i, j, k, Cf)`` is the patch index of each
    boundary face (as for ``mesh.structured_mesh``); ``periodic[d]`` writes
    the two ends of direction d as a cyclic pair named ``cyclic_<d>_lo`` /
    ``cyclic_<d>_hi``; with ``empty_z`` the z ends are one ``frontAndBack``
    empty patch.  The face vertices are ordered so that the area vector
    points out of the owner cell."""
    xs, ys, zs = (np.asarray(a, dtype=np.float64) for a in (xs, ys, zs))
    nx, ny, nz = len(xs) - 1, len(ys) - 1, len(zs) - 1
    pid = lambda i, j, k: i + (nx + 1) * (j + (ny + 1) * k)
    cid = lambda i, j, k: i + nx * (j + ny * k)
    P = np.stack(np.meshgrid(xs, ys, zs, indexing="ij"), -1).transpose(2, 1, 0, 3).reshape(-1, 3)

    def quad(d, i, j, k):
        """vertices of the +d face of cell (i,j,k), counter-clockwise seen from outside"""
        if d == 0:   # x+ face at i+1
            return [pid(i + 1, j, k), pid(i + 1, j + 1, k), pid(i + 1, j + 1, k + 1), pid(i + 1, j, k + 1)]
        if d == 1:
            return [pid(i, j + 1, k), pid(i, j + 1, k + 1), pid(i + 1, j + 1, k + 1), pid(i + 1, j + 1, k)]
        return [pid(i, j, k + 1), pid(i + 1, j, k + 1), pid(i + 1, j + 1, k + 1), pid(i, j + 1, k + 1)]

    def quad_minus(d, i, j, k):
        """the -d face of cell (i,j,k), outward (towards -d)"""
        if d == 0:
            return [pid(i, j, k), pid(i, j, k + 1), pid(i, j + 1, k + 1), pid(i, j + 1, k)]
        if d == 1:
            return [pid(i, j, k), pid(i + 1, j, k), pid(i + 1, j, k + 1), pid(i, j, k + 1)]
        return [pid(i, j, k), pid(i, j + 1, k), pid(i + 1, j + 1, k), pid(i + 1, j, k)]

    internal = []   # (owner, neighbour, verts)
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                c = cid(i, j, k)
                for d, (di, dj, dk) in enumerate(((1, 0, 0), (0, 1, 0), (0, 0, 1))):
                    i2, j2, k2 = i + di, j + dj, k + dk
                    if i2 < nx and j2 < ny and k2 < nz and not (d == 2 and empty_z):
                        internal.append((c, cid(i2, j2, k2), quad(d, i, j, k)))
    internal.sort(key=lambda t: (t[0], t[1]))
    # boundary faces grouped by patch
    names = list(patch_names)
    types = list(patch_types) if patch_types else ["wall"] * len(names)
    groups: Dict[str, List] = {nm: [] for nm in names}
    cyc = []
    for d in range(3):
        if periodic[d]:
            lo, hi = f"cyclic_{'xyz'[d]}_lo", f"cyclic_{'xyz'[d]}_hi"
            groups[lo], groups[hi] = [], []
            cyc.append((lo, hi))
    if empty_z:
        groups["frontAndBack"] = []
    dirs = ((-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1))
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                c = cid(i, j, k)
                for dd, (di, dj, dk) in enumerate(dirs):
                    i2, j2, k2 = i + di, j + dj, k + dk
                    if 0 <= i2 < nx and 0 <= j2 < ny and 0 <= k2 < nz:
                        continue
                    axis, plus = dd // 2, dd % 2 == 1
                    verts = quad(axis, i, j, k) if plus else quad_minus(axis, i, j, k)
                    if axis == 2 and empty_z:
                        groups["frontAndBack"].append((c, verts))
                        continue
                    if periodic[axis]:
                        groups[f"cyclic_{'xyz'[axis]}_{'hi' if plus else 'lo'}"].append((c, (i, j, k), verts))
                        continue
                    fc = P[verts].mean(0)[None]
                    p = int(np.asarray(patch_of(dd, np.array([i]), np.array([j]), np.array([k]), fc)).ravel()[0])
                    if p < 0:
                        continue
                    groups[names[p]].append((c, verts))
    # cyclic halves in matching order (sorted by the transverse cell position)
    for lo, hi in cyc:
        for nm in (lo, hi):
            groups[nm].sort(key=lambda t: (t[1][2], t[1][1], t[1][0]))
            groups[nm] = [(c, v) for c, _, v in groups[nm]]
    order = names + [n for pair in cyc for n in pair] + (["frontAndBack"] if empty_z else [])
    ptype = dict(zip(names, types))
    for lo, hi in cyc:
        ptype[lo] = ptype[hi] = "cyclic"
    if empty_z:
        ptype["frontAndBack"] = "empty"
    allf = [v for _, _, v in internal]
    owner = [o for o, _, _ in internal]
    neigh = [n for _, n, _ in internal]
    bdesc = []
    for nm in order:
        bdesc.append((nm, ptype[nm], len(groups[nm]), len(allf)))
        for c, v in groups[nm]:
            allf.append(v)
            owner.append(c)
    os.makedirs(out_dir, exist_ok=True)
    loc = "constant/polyMesh"
    with open(os.path.join(out_dir, "points"), "w") as f:
        f.write(_header_text("vectorField", "points", loc))
        f.write(f"{len(P)}\n(\n")
        for p in P:
            f.write(f"({_fmt(p[0], prec)} {_fmt(p[1], prec)} {_fmt(p[2], prec)})\n")
        f.write(")\n")
    with open(os.path.join(out_dir, "faces"), "w") as f:
        f.write(_header_text("faceList", "faces", loc))
        f.write(f"{len(allf)}\n(\n")
        for v in allf:
            f.write(f"4({v[0]} {v[1]} {v[2]} {v[3]})\n")
        f.write(")\n")
    note = f"nPoints:{len(P)}  nCells:{nx * ny * nz}  nFaces:{len(allf)}  nInternalFaces:{len(internal)}"
    for obj, lab in (("owner", owner), ("neighbour", neigh)):
        with open(os.path.join(out_dir, obj), "w") as f:
            f.write(_header_text("labelList", obj, loc, note))
            f.write(f"{len(lab)}\n(\n" + "\n".join(str(x) for x in lab) + "\n)\n")
    pair = {}
    for lo, hi in cyc:
        pair[lo], pair[hi] = hi, lo
    with open(os.path.join(out_dir, "boundary"), "w") as f:
        f.write(_header_text("polyBoundaryMesh", "boundary", loc))
        f.write(f"{len(bdesc)}\n(\n")
        for nm, typ, n, s in bdesc:
            f.write(f"    {nm}\n    {{\n        type            {typ};\n")
            if typ == "cyclic":
                f.write(f"        neighbourPatch  {pair[nm]};\n")
            f.write(f"        nFaces          {n};\n        startFace       {s};\n    }}\n")
        f.write(")\n")


# ---------------------------------------------------------------------------
# fields
# ---------------------------------------------------------------------------
_NCOMP = {"volScalarField": 1, "volVectorField": 3, "volSymmTensorField": 6, "volTensorField": 9,
          "surfaceScalarField": 1}


def _value_text(v: np.ndarray, prec: int) -> str:
    v = np.atleast_1d(v)
    if v.size == 1:
        return _fmt(float(v[0]), prec)
    return "(" + " ".join(_fmt(float(x), prec) for x in v) + ")"


def _list_text(a: np.ndarray, nc: int, prec: int) -> str:
    kind = {1: "scalar", 3: "vector", 6: "symmTensor", 9: "tensor"}[nc]
    a = a.reshape(-1, nc) if nc > 1 else a.reshape(-1)
    body = "\n".join(_value_text(x, prec) for x in a)
    return f"nonuniform List<{kind}> \n{len(a)}\n(\n{body}\n)\n"


def write_field(path: str, cls: str, obj: str, internal: np.ndarray, boundary: Dict[str, Tuple[str, Optional[np.ndarray]]],
                dimensions: str = "[0 0 0 0 0 0 0]", time: str = "0", prec: int = 12) -> None:
    """One field file.  ``boundary`` maps each patch name to (type, values or
    None); values are written as a ``value`` entry."""
    nc = _NCOMP[cls]
    with open(path, "w") as f:
        f.write(_header_text(cls, obj, time))
        f.write(f"dimensions      {dimensions};\n\n")
        f.write("internalField   " + _list_text(np.asarray(internal, dtype=np.float64), nc, prec) + ";\n\n")
        f.write("boundaryField\n{\n")
        for nm, (typ, vals) in boundary.items():
            f.write(f"    {nm}\n    {{\n        type            {typ};\n")
            if vals is not None:
                f.write("        value           " + _list_text(np.asarray(vals, dtype=np.float64), nc, prec) + ";\n")
            f.write("    }\n")
        f.write("}\n")


def _parse_values(s: str, nc: int, n: Optional[int]) -> np.ndarray:
    s = s.strip()
    if s.startswith("uniform"):
        v = _numbers(s[len("uniform"):])
        if n is None:
            return v
        return np.tile(v, (n, 1)) if nc > 1 else np.full(n, float(v[0]))
    if s.startswith("nonuniform"):
        cnt, a, b = _list_span(s)
        v = _numbers(s[a:b])
        return v.reshape(cnt, nc) if nc > 1 else v
    raise ValueError(f"cannot read field value {s[:40]!r}")


def read_field(path: str, n_internal: Optional[int] = None) -> Tuple[np.ndarray, Dict[str, Dict]]:
    """(internal values, {patch: {"type": ..., "value": array or None}}).
    A ``uniform`` internal field is expanded to ``n_internal`` entries when
    given."""
    text = _read_text(path)
    cls = _header(text).get("class", "volScalarField")
    nc = _NCOMP.get(cls, 1)
    t = _body(text)
    m = re.search(r"internalField\s+(.*?);\s*\n", t, re.S)
    if not m:
        raise ValueError(f"{path}: no internalField")
    internal = _parse_values(m.group(1), nc, n_internal)
    bf = {}
    mb = re.search(r"boundaryField\s*\{", t)
    if mb:
        depth, i = 1, mb.end()
        start = i
        while depth:
            if t[i] == "{":
                depth += 1
            elif t[i] == "}":
                depth -= 1
            i += 1
        block = t[start:i - 1]
        for pm in re.finditer(r"([\w\"\.\*\|\(\)]+)\s*\{(.*?)\}", block, re.S):
            body = pm.group(2)
            tm = re.search(r"type\s+(\w+)\s*;", body)
            vm = re.search(r"\bvalue\s+(.*?);", body, re.S)
            bf[pm.group(1).strip('"')] = {"type": tm.group(1) if tm else None,
                                          "value": _parse_values(vm.group(1), nc, None) if vm else None}
    return internal, bf


def write_fields(time_dir: str, mesh: Mesh, fields, bc_types: Optional[Dict[str, Dict[str, str]]] = None,
                 prec: int = 12) -> List[str]:
    """Write U, p, phi, theta, tau, eigVals and eigVecs of a ``case.Fields``
    state into ``time_dir`` (OpenFOAM names and classes; eigVals as the
    diagonal tensor the reference stores).  ``bc_types[patch][field]`` names
    the patch type written (default ``calculated``).  Returns the paths."""
    os.makedirs(time_dir, exist_ok=True)
    t = os.path.basename(os.path.normpath(time_dir))
    N = mesh.nCells
    ev = np.zeros((N, 9))
    ev[:, 0], ev[:, 4], ev[:, 8] = fields.eigVals[:, 0], fields.eigVals[:, 1], fields.eigVals[:, 2]
    specs = [("U", "volVectorField", fields.U, fields.Ub, "[0 1 -1 0 0 0 0]"),
             ("p", "volScalarField", fields.p, fields.pb, "[0 2 -2 0 0 0 0]"),
             ("theta", "volSymmTensorField", fields.theta, fields.thetab, "[0 0 0 0 0 0 0]"),
             ("tau", "volSymmTensorField", fields.tau, fields.taub, "[1 -1 -2 0 0 0 0]"),
             ("eigVals", "volTensorField", ev, None, "[0 0 0 0 0 0 0]"),
             ("eigVecs", "volTensorField", fields.eigVecs, None, "[0 0 0 0 0 0 0]")]
    paths = []
    for name, cls, internal, bvals, dims in specs:
        bnd = {}
        for p in mesh.patches:
            typ = (bc_types or {}).get(p.name, {}).get(name, "calculated")
            v = None if bvals is None else np.asarray(bvals)[p.start:p.start + p.size]
            bnd[p.name] = (typ, v)
        path = os.path.join(time_dir, name)
        write_field(path, cls, name, internal, bnd, dims, t, prec)
        paths.append(path)
    # phi: internal faces in OpenFOAM's order; coupled faces go back to their patches
    nI = int(np.sum(mesh.coupled == 0)) if mesh.coupled is not None else mesh.nFaces
    phi_int = np.asarray(fields.phi)
    bnd = {p.name: ("calculated", np.asarray(fields.phib)[p.start:p.start + p.size]) for p in mesh.patches}
    if mesh.coupled is not None:
        keep = mesh.coupled == 0
        src = getattr(mesh, "foamFace", None)
        internal = phi_int[keep]
        if src is not None:
            internal = np.empty(nI)
            internal[src[keep]] = phi_int[keep]
        patches = getattr(mesh, "foamPatches", None)
        if src is not None and patches is not None:
            # each cyclic patch face gets the flux out of its own cell: the
            # pair's flux on the owner's face, minus it on the partner's face
            face_phi = {}
            cf = np.nonzero(~keep)[0]
            for f in cf:
                face_phi[int(src[f])] = phi_int[f]
                face_phi[int(mesh.foamPartner[f])] = -phi_int[f]
            for pd in patches:
                if pd.get("type") == "cyclic":
                    s0, n0 = int(pd["startFace"]), int(pd["nFaces"])
                    bnd[pd["name"]] = ("cyclic", np.array([face_phi[i] for i in range(s0, s0 + n0)]))
        else:
            bnd["coupled"] = ("cyclic", phi_int[~keep])
    else:
        internal = phi_int
        src = getattr(mesh, "foamFace", None)
        if src is not None:
            internal = np.empty(nI)
            internal[src] = phi_int
    path = os.path.join(time_dir, "phi")
    write_field(path, "surfaceScalarField", "phi", internal, bnd, "[0 3 -1 0 0 0 0]", t, prec)
    paths.append(path)
    return paths
