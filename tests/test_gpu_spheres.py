"""Rigid spheres with no-slip bounce-back and virtual particles in cut cells.

The reference's only bounce-back surfaces are the planar walls of -DNOSLIP
(streaming reflection, src/libcilia/mpcd.cpp:346-376; virtual particles in
the wall layers, mpcd.cpp:175-198); the engine extends both rules to rigid
spheres (mpcd_set_rigid_spheres).  Its parity is pinned three ways:

  * planar limit: two held spheres of radius 1e7 whose surfaces pass through
    z = 0 and z = Lz - 1 stand for the no-slip walls; on the same injected
    randomness (grid shifts, Gamma variates, rotation axes and the virtual
    particles' momenta) the fluid of the lower half matches the walls path:
    velocities to round-off, positions exactly except for the reflected
    particles, which the surface's height over the plane (at most 1.6e-6
    across the box) moves by up to 1e-3 for grazing incidence;
  * conservation: a free sphere exchanges momentum with the fluid only, so
    fluid + sphere momentum stays constant to round-off (float64 sums;
    float32 split: to its float rounding);
  * Stokes drag: a held sphere in a periodic box of fluid driven by a body
    force g; in the steady state the mean force on the sphere balances the
    force on the fluid (N g), and the drag coefficient F / (6 pi eta R U),
    U the mean fluid velocity, agrees with Hasimoto's periodic-array factor
    K(c) = 1 / (1 - 1.7601 c^(1/3) + c - 1.5593 c^2) (c the sphere's volume
    fraction) within 15 %, eta = 8.70 the SRD viscosity of h = 0.1,
    rho = 10, alpha = 130 degrees, kT = 1 (the Poiseuille test measures it).
"""
import numpy as np
import pytest

import cilia_gpu as cg

pytestmark = pytest.mark.gpu


def periodic_diff(a, b, L):
    d = a - b
    L = np.asarray(L, dtype=float)
    return d - np.round(d / L) * L


def fluid_outside(L, spheres, rho=10, seed=1):
    """rho particles per cell, uniform over the box minus the spheres (nearest
    images), Maxwell-Boltzmann velocities at kT = 1 with zero mean."""
    rng = np.random.default_rng(seed)
    L = np.asarray(L, dtype=float)
    n = int(rho * np.prod(L))
    pos = rng.uniform(0, 1, (2 * n, 3)) * L
    keep = np.ones(len(pos), dtype=bool)
    for sp in spheres:
        d = periodic_diff(pos, np.asarray(sp["center"], dtype=float), L)
        keep &= (d ** 2).sum(axis=1) > sp["radius"] ** 2
    pos = pos[keep]
    vol = np.prod(L) - sum(4.0 / 3.0 * np.pi * sp["radius"] ** 3 for sp in spheres)
    pos = pos[: int(rho * vol)]
    vel = rng.normal(size=pos.shape)
    vel -= vel.mean(axis=0)
    return pos, vel


def test_planar_limit_matches_walls_path():
    L = (8, 8, 12)
    R = 1.0e7
    rng = np.random.default_rng(4)
    n = 8 * 8 * 11 * 10
    pos = rng.uniform(0, 1, (n, 3)) * np.array([8.0, 8.0, 11.0])
    vel = rng.normal(size=(n, 3))
    walls = cg.Engine(L, tstep=0.1, ststep=0.002, walls=cg.WALLS_NOSLIP)
    sph = cg.Engine(L, tstep=0.1, ststep=0.002)
    sph.set_rigid_spheres([dict(center=(4.0, 4.0, -R), radius=R), dict(center=(4.0, 4.0, 11.0 + R), radius=R)])
    a0 = np.array([0.31, 0.62, 0.47])
    for e in (walls, sph):
        e.set_fluid(pos, vel)
        e.shift = a0
    ncell = 8 * 8 * 12
    for k in range(2):
        shift = rng.uniform(0, 1, 3)
        gamma = rng.gamma(13.5, size=ncell)
        axis = rng.normal(size=(ncell, 3))
        axis /= np.linalg.norm(axis, axis=1)[:, None]
        virt = rng.normal(size=(ncell, 3)) * 2.0
        for e in (walls, sph):
            e.step(shift, gamma, axis, virt)
    pw, vw = walls.fluid()
    ps, vs = sph.fluid()
    low = pw[:, 2] < 6.0
    assert low.sum() > 2000
    dp = np.abs(periodic_diff(ps[low], pw[low], L)).max(axis=1)
    dv = np.abs(vs[low] - vw[low]).max()
    # no-slip bounce-back reverses the velocity whatever the surface's tilt:
    # velocities agree to round-off; a reflected particle's position moves by
    # 2 |v| dz / |v_z| with dz <= (4^2 + 4^2) / (2 R) = 1.6e-6 the height of
    # the curved surface over the plane, large only for grazing particles;
    # every other particle is untouched by the curvature
    assert dv < 1e-12, dv
    assert dp.max() < 1e-3, dp.max()
    assert np.mean(dp < 1e-12) > 0.95, np.mean(dp < 1e-12)
    # the bottom surface did reflect particles in both
    assert np.all(ps[low, 2] >= -1e-6)


@pytest.mark.parametrize("precision", [cg.MPCD_FP64, cg.MPCD_FP32])
def test_free_sphere_conserves_momentum(precision):
    L = (16, 16, 16)
    R = 3.0
    mass = 10 * 4.0 / 3.0 * np.pi * R ** 3
    sp = dict(center=(8.0, 8.0, 8.0), radius=R, mass=mass, velocity=(0.05, -0.02, 0.01), omega=(0.0, 0.0, 0.01))
    pos, vel = fluid_outside(L, [sp], seed=2)
    e = cg.Engine(L, tstep=0.1, ststep=0.002, precision=precision, seed=7)
    e.set_fluid(pos, vel)
    e.set_rigid_spheres([sp])
    _, v0 = e.fluid()
    P0 = v0.sum(axis=0) + mass * np.array(sp["velocity"])
    e.run(100)
    (s1,), ft = e.rigid_spheres()
    _, v1 = e.fluid()
    P1 = v1.sum(axis=0) + mass * s1["velocity"]
    moved = np.linalg.norm(periodic_diff(s1["center"], np.array(sp["center"]), L))
    assert moved > 0.1  # it moved, carried by its own momentum and the fluid's
    assert np.abs(s1["velocity"] - np.array(sp["velocity"])).max() > 1e-4  # and exchanged momentum
    tol = 1e-9 * np.abs(P0).max() + 1e-9 if precision == cg.MPCD_FP64 else 5e-3
    assert np.abs(P1 - P0).max() < tol, (P1 - P0)
    # no fluid particle ends inside the sphere
    p1, _ = e.fluid()
    d = periodic_diff(p1, s1["center"], L)
    assert (np.sqrt((d ** 2).sum(axis=1)) > R - 1e-6).all()


def test_held_sphere_stokes_drag():
    """Stokes drag of a held sphere in a periodic box, three runs (the ratio
    below varies by about 7 % from run to run: the mean fluid velocity U over
    100 samples is noisy), their mean within 15 % of Hasimoto's factor."""
    L = (16, 16, 16)
    R = 3.0
    g = 0.001
    c = 4.0 / 3.0 * np.pi * R ** 3 / np.prod(L)
    K = 1.0 / (1.0 - 1.7601 * c ** (1.0 / 3.0) + c - 1.5593 * c * c)
    eta = 8.70
    ratios = []
    for run in range(3):
        sp = dict(center=(8.0, 8.0, 8.0), radius=R)
        pos, vel = fluid_outside(L, [sp], seed=3 + run)
        nf = len(pos)
        e = cg.Engine(L, tstep=0.1, ststep=0.002, precision=cg.MPCD_FP32, seed=11 + run, gravity=g)
        e.set_fluid(pos, vel)
        e.set_rigid_spheres([sp])
        e.run(4000)
        e.reset_sphere_forces()
        us = []
        for _ in range(100):
            e.run(40)
            us.append(e.observables()["momentum"][0])
        (s1,), ft = e.rigid_spheres()
        F = ft[0, 0]
        U = float(np.mean(us))
        # momentum balance of the steady state: the sphere holds the fluid against the body force
        assert abs(F - nf * g) < 0.05 * nf * g, (F, nf * g)
        ratios.append(F / (6 * np.pi * eta * R * U) / K)
        # the held sphere did not move
        assert np.array_equal(s1["center"], np.array(sp["center"])) and not s1["velocity"].any()
        e.close()
    print("stokes", dict(K=K, ratios=ratios))
    assert abs(np.mean(ratios) - 1.0) < 0.15, ratios


def test_rigid_sphere_arguments_rejected():
    e = cg.Engine((8, 8, 8))
    with pytest.raises(cg.MpcdError):
        e.set_rigid_spheres([dict(center=(1, 1, 1), radius=-1.0)])
    with pytest.raises(cg.MpcdError):
        e.set_rigid_spheres([dict(center=(np.nan, 1, 1), radius=1.0)])
    with pytest.raises(cg.MpcdError):
        e.set_rigid_spheres([dict(center=(1, 1, 1), radius=1.0)] * 5)
    e.set_rigid_spheres([dict(center=(9.5, -0.5, 4.0), radius=1.0)])  # wrapped into the box
    (s,), _ = e.rigid_spheres()
    assert np.allclose(s["center"], [1.5, 7.5, 4.0])
    e.set_rigid_spheres([])
