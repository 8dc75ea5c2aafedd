"""OpenFOAM case I/O on the CPU: polyMesh files written for structured grids
read back into the same LDU mesh the generator builds (addressing, geometry,
patches, cyclic pairs), primitiveMesh geometry on distorted cells, field
files that read back what was written, and an oracle step on a mesh read
from polyMesh files equal to the step on the generated mesh."""
import os

import numpy as np
import pytest

from rheotool_gb300 import foam_io
from rheotool_gb300.case import cavity_case, periodic_channel_case, periodic_channel_state
from rheotool_gb300.mesh import (XM, XP, YM, YP, ZM, ZP, cavity_mesh, graded_nodes, periodic_channel_mesh,
                                 structured_mesh, two_sided_nodes)


def _same_mesh(a, b, tol=1e-12):
    assert a.nCells == b.nCells and a.nFaces == b.nFaces and a.nBFaces == b.nBFaces
    assert np.array_equal(a.owner, b.owner) and np.array_equal(a.neighbour, b.neighbour)
    for name in ("Sf", "magSf", "w", "deltaCoeffs", "C", "V"):
        x, y = getattr(a, name), getattr(b, name)
        assert np.allclose(x, y, rtol=tol, atol=tol * np.abs(y).max()), name
    for name in ("bCell",):
        assert np.array_equal(getattr(a, name), getattr(b, name)), name
    for name in ("bSf", "bmagSf", "bCf", "bDelta"):
        x, y = getattr(a, name), getattr(b, name)
        assert np.allclose(x, y, rtol=tol, atol=tol * np.abs(y).max()), name
    assert [(p.name, p.start, p.size) for p in a.patches] == [(p.name, p.start, p.size) for p in b.patches]
    assert np.array_equal(a.solveDir, b.solveDir)


def _cavity_patch_of(d, i, j, k, Cf):
    if d == YP:
        return np.zeros(i.size, np.int64)
    return np.ones(i.size, np.int64)


def test_cavity_polymesh_roundtrip(tmp_path):
    n = 6
    ref = cavity_mesh(n)
    xs = graded_nodes(0.0, 1.0, n)
    foam_io.write_structured_polymesh(str(tmp_path), xs, xs, np.array([-0.5, 0.5]), _cavity_patch_of,
                                      ["movingLid", "fixedWalls"], empty_z=True)
    m = foam_io.read_polymesh(str(tmp_path))
    m.check()
    _same_mesh(m, ref)
    assert list(m.solveDir) == [1, 1, 0]


def test_graded_3d_box_roundtrip(tmp_path):
    xs = graded_nodes(0.0, 2.0, 5, 3.0)
    ys = two_sided_nodes(-1.0, 1.0, 4, 2.0)
    zs = graded_nodes(0.0, 1.0, 3, 0.5)

    def patch_of(d, i, j, k, Cf):
        return np.full(i.size, {XM: 0, XP: 1}.get(d, 2), np.int64)

    names = ["inlet", "outlet", "walls"]
    ref = structured_mesh(xs, ys, zs, patch_of, names)
    foam_io.write_structured_polymesh(str(tmp_path), xs, ys, zs, patch_of, names, ["patch", "patch", "wall"])
    m = foam_io.read_polymesh(str(tmp_path))
    _same_mesh(m, ref)


def test_periodic_channel_polymesh_roundtrip(tmp_path):
    ref = periodic_channel_mesh(5, 4, 3, L=2.0, H=1.0, depth=1.0, wall_ratio=2.0)
    xs = graded_nodes(0.0, 2.0, 5)
    ys = two_sided_nodes(-1.0, 1.0, 4, 2.0)
    zs = graded_nodes(0.0, 1.0, 3)
    foam_io.write_structured_polymesh(str(tmp_path), xs, ys, zs, lambda d, i, j, k, Cf: np.zeros(i.size, np.int64),
                                      ["walls"], periodic=(True, False, True))
    m = foam_io.read_polymesh(str(tmp_path))
    m.check()
    _same_mesh(m, ref)
    assert np.array_equal(m.coupled, ref.coupled)
    assert np.allclose(m.delta, ref.delta, atol=1e-14)


def test_distorted_cells_geometry(tmp_path):
    """Moved interior points: cells stay closed, the volumes add up to the box,
    and a linear field's Gauss gradient (face values from the geometry) is
    exact only through the area vectors, which are checked to close."""
    n = 4
    xs = graded_nodes(0.0, 1.0, n)
    foam_io.write_structured_polymesh(str(tmp_path), xs, xs, xs, lambda d, i, j, k, Cf: np.zeros(i.size, np.int64),
                                      ["walls"])
    pts = foam_io.read_vector_list(os.path.join(str(tmp_path), "points"))
    rng = np.random.default_rng(3)
    inner = np.all((pts > 1e-9) & (pts < 1 - 1e-9), axis=1)
    pts[inner] += 0.05 / n * rng.uniform(-1, 1, size=(int(inner.sum()), 3))
    with open(os.path.join(str(tmp_path), "points"), "w") as f:
        f.write(foam_io._header_text("vectorField", "points", "constant/polyMesh"))
        f.write(f"{len(pts)}\n(\n" + "\n".join("(" + " ".join(f"{float(x):.17g}" for x in p) + ")" for p in pts) + "\n)\n")
    m = foam_io.read_polymesh(str(tmp_path))
    m.check()
    assert abs(m.V.sum() - 1.0) < 1e-12
    assert np.all(m.V > 0) and np.all((m.w > 0) & (m.w < 1))


def test_field_write_read_roundtrip(tmp_path):
    case = periodic_channel_case(periodic_channel_mesh(4, 4, 3, L=2.0, depth=1.0), Wi=2.0)
    f = periodic_channel_state(case, sigma=0.1, seed=4)
    paths = foam_io.write_fields(str(tmp_path / "0.5"), case.mesh, f, prec=17)
    assert {os.path.basename(p) for p in paths} == {"U", "p", "theta", "tau", "eigVals", "eigVecs", "phi"}
    U, bU = foam_io.read_field(str(tmp_path / "0.5" / "U"))
    assert np.array_equal(U, f.U)
    assert np.array_equal(bU["walls"]["value"], f.Ub)
    th, _ = foam_io.read_field(str(tmp_path / "0.5" / "theta"))
    assert np.array_equal(th, f.theta)
    ev, _ = foam_io.read_field(str(tmp_path / "0.5" / "eigVals"))
    assert np.array_equal(ev[:, [0, 4, 8]], f.eigVals)
    phi, bphi = foam_io.read_field(str(tmp_path / "0.5" / "phi"))
    keep = case.mesh.coupled == 0
    assert np.array_equal(phi, f.phi[keep]) and np.array_equal(bphi["coupled"]["value"], f.phi[~keep])


def test_read_uniform_field(tmp_path):
    p = tmp_path / "p"
    p.write_text('FoamFile\n{\n version 2.0;\n format ascii;\n class volScalarField;\n object p;\n}\n'
                 '// comment\ndimensions [0 2 -2 0 0 0 0];\ninternalField   uniform 0;\n'
                 'boundaryField\n{\n    movingLid\n    {\n        type zeroGradient;\n    }\n'
                 '    fixedWalls { type fixedValue; value uniform 2.5; }\n}\n')
    v, b = foam_io.read_field(str(p), n_internal=7)
    assert v.shape == (7,) and np.all(v == 0.0)
    assert b["movingLid"]["type"] == "zeroGradient" and b["movingLid"]["value"] is None
    assert np.allclose(b["fixedWalls"]["value"], [2.5])


def test_oracle_step_on_read_mesh_equals_generated(tmp_path):
    from oracle.pyoracle import Oracle
    n = 8
    xs = graded_nodes(0.0, 1.0, n)
    foam_io.write_structured_polymesh(str(tmp_path), xs, xs, np.array([-0.5, 0.5]), _cavity_patch_of,
                                      ["movingLid", "fixedWalls"], empty_z=True)
    read = foam_io.read_polymesh(str(tmp_path))
    a, b = Oracle(cavity_case(n)), Oracle(cavity_case(n, mesh=read))
    a.step(3)
    b.step(3)
    for name in ("U", "p", "theta", "tau", "phi"):
        x, y = getattr(b.f, name), getattr(a.f, name)
        assert np.linalg.norm(x - y) <= 1e-11 * max(np.linalg.norm(y), 1e-300), name


def test_cyclic_phi_written_on_both_patches(tmp_path):
    """A periodic mesh read from polyMesh files writes phi in OpenFOAM's
    layout: internal faces in their order, each cyclic patch face with the
    flux out of its own cell (the two halves of a pair opposite)."""
    xs = graded_nodes(0.0, 2.0, 5)
    ys = two_sided_nodes(-1.0, 1.0, 4, 2.0)
    zs = graded_nodes(0.0, 1.0, 3)
    foam_io.write_structured_polymesh(str(tmp_path / "mesh"), xs, ys, zs,
                                      lambda d, i, j, k, Cf: np.zeros(i.size, np.int64), ["walls"],
                                      periodic=(True, False, True))
    m = foam_io.read_polymesh(str(tmp_path / "mesh"))
    case = periodic_channel_case(m, Wi=2.0)
    f = periodic_channel_state(case)
    foam_io.write_fields(str(tmp_path / "0"), m, f, prec=17)
    phi, b = foam_io.read_field(str(tmp_path / "0" / "phi"))
    keep = m.coupled == 0
    assert phi.size == int(keep.sum())
    lo, hi = b["cyclic_x_lo"]["value"], b["cyclic_x_hi"]["value"]
    assert np.allclose(lo, -hi) and np.abs(hi).max() > 0          # the flow leaves at x = L, enters at x = 0
    assert np.all(hi > 0)
    zl, zh = b["cyclic_z_lo"]["value"], b["cyclic_z_hi"]["value"]
    assert np.allclose(zl, 0.0) and np.allclose(zh, 0.0)           # no spanwise flow


def _write_binary(path, cls, obj, arrays):
    hdr = ('FoamFile\n{\n    version 2.0;\n    format binary;\n    arch "LSB;label=32;scalar=64";\n'
           f'    class {cls};\n    location "constant/polyMesh";\n    object {obj};\n}}\n\n')
    with open(path, "wb") as f:
        f.write(hdr.encode())
        for a in arrays:
            f.write(f"{len(a)}\n(".encode())
            f.write(np.ascontiguousarray(a).tobytes())
            f.write(b")\n\n")


def test_binary_polymesh_reads_like_ascii(tmp_path):
    """A polyMesh written in OpenFOAM's binary format (labels int32, scalars
    float64, faces as a faceCompactList) reads into the same mesh as the
    ASCII files."""
    ascii_dir, bin_dir = str(tmp_path / "a"), str(tmp_path / "b")
    xs = graded_nodes(0.0, 1.0, 5, 2.0)
    foam_io.write_structured_polymesh(ascii_dir, xs, xs, xs, lambda d, i, j, k, Cf: np.zeros(i.size, np.int64),
                                      ["walls"])
    ref = foam_io.read_polymesh(ascii_dir)
    os.makedirs(bin_dir)
    pts = foam_io.read_vector_list(os.path.join(ascii_dir, "points"))
    faces = foam_io.read_faces(os.path.join(ascii_dir, "faces"))
    own = foam_io.read_label_list(os.path.join(ascii_dir, "owner")).astype(np.int32)
    nei = foam_io.read_label_list(os.path.join(ascii_dir, "neighbour")).astype(np.int32)
    offs = np.concatenate([[0], np.cumsum([len(f) for f in faces])]).astype(np.int32)
    lab = np.concatenate(faces).astype(np.int32)
    _write_binary(os.path.join(bin_dir, "points"), "vectorField", "points", [pts.astype(np.float64)])
    _write_binary(os.path.join(bin_dir, "faces"), "faceCompactList", "faces", [offs, lab])
    _write_binary(os.path.join(bin_dir, "owner"), "labelList", "owner", [own])
    _write_binary(os.path.join(bin_dir, "neighbour"), "labelList", "neighbour", [nei])
    with open(os.path.join(ascii_dir, "boundary")) as f, open(os.path.join(bin_dir, "boundary"), "w") as g:
        g.write(f.read())
    m = foam_io.read_polymesh(bin_dir)
    _same_mesh(m, ref, tol=0.0 + 1e-15)


def test_mesh_quality():
    m = periodic_channel_mesh(5, 4, 3, L=2.0, depth=1.0)
    q = foam_io.mesh_quality(m)
    assert q["nonOrthogonality"] < 1e-9 and q["skewness"] < 1e-9


def test_mesh_quality_of_distorted_cells(tmp_path):
    n = 3
    xs = graded_nodes(0.0, 1.0, n)
    foam_io.write_structured_polymesh(str(tmp_path), xs, xs, xs, lambda d, i, j, k, Cf: np.zeros(i.size, np.int64),
                                      ["walls"])
    pts = foam_io.read_vector_list(os.path.join(str(tmp_path), "points"))
    inner = np.all((pts > 1e-9) & (pts < 1 - 1e-9), axis=1)
    pts[inner] += 0.05
    with open(os.path.join(str(tmp_path), "points"), "w") as f:
        f.write(foam_io._header_text("vectorField", "points", "constant/polyMesh"))
        f.write(f"{len(pts)}\n(\n" + "\n".join("(" + " ".join(f"{float(x):.17g}" for x in p) + ")" for p in pts) + "\n)\n")
    q = foam_io.mesh_quality(foam_io.read_polymesh(str(tmp_path)))
    assert q["nonOrthogonality"] > 1.0
