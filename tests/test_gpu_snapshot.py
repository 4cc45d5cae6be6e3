"""Lossless snapshots (mpcd_snapshot / mpcd_restore): a handle's whole state
as host bytes, restored into a fresh handle of the same box.

  * Right after the restore the state is the snapshotted one bit for bit
    (fluid, beads, grid shift, time).
  * The restored run continues the original: both run the same free steps
    (the generator is keyed by seed and step counter, both restored); they
    differ only by the order of the atomic additions into the cell sums, so
    float64 positions agree to 1e-9 after 3 steps of a swimmer (beads and
    fluid), split precision for 99.9 % of the particles to 1e-4.
  * A snapshot of another box, precision or time step is refused.
"""
import numpy as np
import pytest

import cilia_gpu as cg
import simcfg

pytestmark = pytest.mark.gpu


def periodic_diff(a, b, L):
    d = a - b
    L = np.asarray(L, dtype=float)
    return d - np.round(d / L) * L


@pytest.mark.parametrize("precision", [cg.MPCD_FP64, cg.MPCD_FP32])
def test_snapshot_restore_continues_the_run(precision):
    cfg = simcfg.swimmer_config(16, radius=4.0, n_cilia=10, rodlength=8, seed=3, ststep=0.002)
    text = simcfg.dumps(cfg)
    a = cg.Sim(text, precision=precision, ststep=0.002, seed=9)
    a.engine.set_rigid_spheres([dict(center=(2.0, 2.0, 2.0), radius=1.0, mass=40.0, velocity=(0.01, 0.0, 0.0))])
    a.engine.run(5)
    snap = a.engine.snapshot()
    p0, v0 = a.engine.fluid()
    b0, bv0 = a.beads()
    t0, s0 = a.engine.time, a.engine.shift
    a.engine.run(3)
    pa, va = a.engine.fluid()
    ba, _ = a.beads()
    (sa,), _ = a.engine.rigid_spheres()
    # a fresh handle with the same box and steps: no beads, no fluid until restored
    e = cg.Engine((16, 16, 16), tstep=0.1, ststep=0.002, precision=precision, seed=1)
    e.restore(snap)
    p1, v1 = e.fluid()
    b1, bv1 = e.beads(a.nbeads)
    assert np.array_equal(p1, p0) and np.array_equal(v1, v0)
    assert np.array_equal(b1, b0) and np.array_equal(bv1, bv0)
    assert e.time == t0 and np.array_equal(e.shift, s0)
    e.run(3)
    pb, vb = e.fluid()
    bb, _ = e.beads(a.nbeads)
    (sb,), _ = e.rigid_spheres()
    L = (16, 16, 16)
    dp = np.abs(periodic_diff(pb, pa, L)).max(axis=1)
    dv = np.abs(vb - va).max(axis=1)
    if precision == cg.MPCD_FP64:
        assert dp.max() < 1e-9 and dv.max() < 1e-8, (dp.max(), dv.max())
        assert np.abs(bb - ba).max() < 1e-9
        assert np.abs(sb["center"] - sa["center"]).max() < 1e-9
    else:
        assert np.mean(dp < 1e-4) > 0.999 and np.mean(dv < 1e-4) > 0.999
        assert np.abs(bb - ba).max() < 1e-3
    assert e.time == a.engine.time
    a.close()


def test_restore_refuses_another_box():
    e = cg.Engine((8, 8, 8), tstep=0.1, ststep=0.002)
    rng = np.random.default_rng(1)
    e.set_fluid(rng.uniform(0, 8, (5120, 3)), rng.normal(size=(5120, 3)))
    snap = e.snapshot()
    for kw in (dict(L=(8, 8, 10)), dict(L=(8, 8, 8), precision=cg.MPCD_FP32), dict(L=(8, 8, 8), ststep=0.001)):
        L = kw.pop("L")
        f = cg.Engine(L, tstep=0.1, **{"ststep": 0.002, **kw})
        with pytest.raises(cg.MpcdError, match="restore"):
            f.restore(snap)
    f = cg.Engine((8, 8, 8), tstep=0.1, ststep=0.002)
    with pytest.raises(cg.MpcdError):
        f.restore(snap[:100])
    with pytest.raises(cg.MpcdError):
        f.restore(b"X" * len(snap))
