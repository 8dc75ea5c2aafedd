"""Cyclic (periodic) patches and the body-force-driven periodic channel, on
the CPU: the mesh's coupled faces, the oracle's treatment of them, and known
answers of the periodic channel (translation invariance, the laminar
Oldroyd-B velocity profile, the force balance at the walls)."""
import numpy as np
import pytest

from rheotool_gb300.case import (lognormal_conformation, periodic_channel_case, periodic_channel_state)
from rheotool_gb300.mesh import periodic_channel_mesh

from oracle.pyoracle import Oracle


def test_periodic_mesh_coupled_faces():
    m = periodic_channel_mesh(6, 5, 4, L=3.0, H=1.0, depth=2.0)
    m.check()                                   # closed cells, upper-triangular order
    nx, ny, nz = m.shape
    assert m.nCells == nx * ny * nz
    assert m.coupled.sum() == ny * nz + nx * ny   # one face per x pair and per z pair
    assert [p.name for p in m.patches] == ["walls"] and m.nBFaces == 2 * nx * nz
    ij = m.cellIJK
    c = np.nonzero(m.coupled)[0]
    o, n = m.owner[c], m.neighbour[c]
    dx = ij[n] - ij[o]
    xw = dx[:, 0] == nx - 1
    zw = dx[:, 2] == nz - 1
    assert np.all(xw ^ zw)
    # across a cyclic face the neighbour sits one cell beyond the owner's end
    assert np.allclose(m.delta[c[xw]], [-3.0 / nx, 0, 0])
    assert np.allclose(m.delta[c[zw]], [0, 0, -2.0 / nz])
    assert np.allclose(m.deltaCoeffs[c[xw]], nx / 3.0)
    assert np.allclose(m.w[c], 0.5)
    # the other faces: delta = C_N - C_P
    k = np.nonzero(m.coupled == 0)[0]
    assert np.allclose(m.delta[k], m.C[m.neighbour[k]] - m.C[m.owner[k]])


def test_lognormal_conformation_is_consistent():
    th, ev, vv = lognormal_conformation(500, sigma=0.1, seed=7)
    assert np.all(np.diff(ev, axis=1) >= 0)
    R = vv.reshape(-1, 3, 3)
    assert np.allclose(np.einsum("nji,njk->nik", R, R), np.eye(3)[None], atol=1e-13)
    T = np.einsum("nij,nj,nkj->nik", R, np.log(ev), R)
    th2 = np.stack([T[:, 0, 0], T[:, 0, 1], T[:, 0, 2], T[:, 1, 1], T[:, 1, 2], T[:, 2, 2]], axis=1)
    assert np.allclose(th, th2, atol=1e-14)
    mu = np.log(ev).ravel()
    assert abs(mu.std() - 0.1) < 0.01 and abs(mu.mean()) < 0.01
    th3, _, _ = lognormal_conformation(500, sigma=0.1, seed=7)
    assert np.array_equal(th, th3)             # seeded


def _uniform_conformation(case, seed=5):
    """The laminar profile with one non-degenerate conformation in every cell
    (from exactly theta = 0 the log-conformation update divides round-off by
    round-off in decomposeGradU and loses any symmetry)."""
    f = periodic_channel_state(case, sigma=0.0)
    th, ev, vv = lognormal_conformation(1, sigma=0.1, seed=seed)
    N = case.mesh.nCells
    f.theta[:] = th
    f.eigVals[:] = ev
    f.eigVecs[:] = vv
    R = vv.reshape(3, 3)
    A = R @ np.diag(ev[0]) @ R.T
    c = case.model.etaP / case.model.lambda_
    T = c * (A - np.eye(3))
    f.tau[:] = [T[0, 0], T[0, 1], T[0, 2], T[1, 1], T[1, 2], T[2, 2]]
    f.thetab[:] = f.theta[case.mesh.bCell]
    f.taub[:] = f.tau[case.mesh.bCell]
    assert f.theta.shape == (N, 6)
    return f


def test_periodic_channel_is_translation_invariant():
    """From an x- and z-independent state the solution must stay independent
    of x and z: any error in the cyclic coupling shows up at the ends of the
    box."""
    mesh = periodic_channel_mesh(5, 8, 4, L=2.0, depth=1.0, wall_ratio=2.0)
    case = periodic_channel_case(mesh, model="Oldroyd-BLog", Wi=0.5, beta=0.5, dt=5e-3)
    o = Oracle(case, fields=_uniform_conformation(case))
    o.step(6)
    nx, ny, nz = mesh.shape
    U = o.f.U.reshape(nz, ny, nx, 3)
    assert np.abs(U[..., 0]).max() > 1e-2
    assert np.abs(U - U[:1, :, :1]).max() <= 1e-9 * np.abs(U).max()
    # cell continuity: the fluxes through the cyclic faces balance as the others
    div = np.zeros(mesh.nCells)
    np.add.at(div, mesh.owner, o.f.phi)
    np.add.at(div, mesh.neighbour, -o.f.phi)
    np.add.at(div, mesh.bCell, o.f.phib)
    assert np.abs(div).max() < 1e-9 * np.abs(o.f.phi).max()
    th = o.f.theta.reshape(nz, ny, nx, 6)
    assert np.abs(th - th[:1, :, :1]).max() <= 1e-9 * np.abs(th).max()


def test_periodic_channel_oldroydb_steady_profile():
    """Steady Oldroyd-B channel flow under a body force: the velocity is the
    Newtonian parabola of eta0 = etaS + etaP with the force's mean velocity,
    and tau_xy = etaP du/dy; the wall shear balances the body force."""
    mesh = periodic_channel_mesh(3, 24, 3, L=1.0, depth=1.0, wall_ratio=1.0)
    case = periodic_channel_case(mesh, model="Oldroyd-BLog", Wi=0.05, beta=0.5, rho=0.01, dt=2e-3)
    case.solverP.tolerance = 1e-10
    o = Oracle(case)
    o.step(300)                                  # 12 relaxation times
    nx, ny, nz = mesh.shape
    y = mesh.C[:ny * nx:nx, 1]
    u = o.f.U[:ny * nx:nx, 0]
    exact = 1.5 * (1.0 - y ** 2)
    assert np.max(np.abs(u - exact)) < 5e-3 * 1.5
    txy = o.f.tau[:ny * nx:nx, 1]
    assert np.max(np.abs(txy - 0.5 * (-3.0 * y))) < 3e-2
    # force balance: body force on the fluid = wall shear (solvent + polymer)
    g = case.bodyForce[0]
    drive = case.model.rho * g * mesh.V.sum()
    b = np.arange(mesh.nBFaces)
    wall = case.model.etaS * (o.f.U[mesh.bCell[b], 0] * mesh.bDelta * mesh.bmagSf).sum() \
        + case.model.etaP * (o.f.U[mesh.bCell[b], 0] * mesh.bDelta * mesh.bmagSf).sum()
    assert abs(wall - drive) < 2e-2 * drive


def test_periodic_channel_state_ptt():
    mesh = periodic_channel_mesh(4, 6, 3, L=2.0, depth=1.0)
    case = periodic_channel_case(mesh, Wi=2.0)
    f = periodic_channel_state(case, sigma=0.1, seed=3)
    A = np.einsum("nij,nj,nkj->nik", f.eigVecs.reshape(-1, 3, 3), f.eigVals, f.eigVecs.reshape(-1, 3, 3))
    c = case.model.etaP / case.model.lambda_
    assert np.allclose(f.tau[:, 0], c * (A[:, 0, 0] - 1.0))
    assert np.allclose(f.tau[:, 1], c * A[:, 0, 1])
    # the flux field carries the profile's flow rate through every x section
    o = Oracle(case, fields=f.copy())
    o.step(1)
    assert np.isfinite(o.f.U).all() and np.isfinite(o.f.theta).all()


def test_inner_iterations_steady_profile_and_default():
    """SIMPLE nInIter: 0 and 1 are the same step (bit for bit); with 2 inner
    iterations per step the steady Oldroyd-B channel reaches the same laminar
    profile."""
    mesh = periodic_channel_mesh(3, 24, 3, L=1.0, depth=1.0, wall_ratio=1.0)
    a = periodic_channel_case(mesh, model="Oldroyd-BLog", Wi=0.05, beta=0.5, rho=0.01, dt=2e-3)
    b = periodic_channel_case(mesh, model="Oldroyd-BLog", Wi=0.05, beta=0.5, rho=0.01, dt=2e-3)
    b.nInIter = 0
    oa, ob = Oracle(a), Oracle(b)
    oa.step(3)
    ob.step(3)
    assert np.array_equal(oa.f.U, ob.f.U) and np.array_equal(oa.f.theta, ob.f.theta)
    c = periodic_channel_case(mesh, model="Oldroyd-BLog", Wi=0.05, beta=0.5, rho=0.01, dt=2e-3)
    c.nInIter = 2
    c.solverP.tolerance = 1e-10
    oc = Oracle(c)
    oc.step(3)
    assert not np.array_equal(oc.f.U, oa.f.U)       # the inner iteration changes the transient
    oc.step(297)
    nx, ny, nz = mesh.shape
    y = mesh.C[:ny * nx:nx, 1]
    u = oc.f.U[:ny * nx:nx, 0]
    assert np.max(np.abs(u - 1.5 * (1.0 - y ** 2))) < 5e-3 * 1.5
