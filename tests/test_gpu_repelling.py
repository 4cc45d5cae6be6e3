"""Contact forces between cilia (the reference's -DREPELLING=eps,
src/libcilia/globalforces.cpp:22-95) against the C oracle's restatement.

The reference's own -DREPELLING build does not compile (its GlobalForces
names a `cilias` list it does not declare), so there is no reference fixture;
the oracle restates the algorithm over the cilia in object order and is the
pin.  A small sphere crowded with 40 cilia of 10 beads keeps neighbouring
cilia within the 1.5 cutoff; with eps = 1000 thousands of section pairs
interact in two MPC steps (counted by the oracle).  On the same injected
randomness the GPU's float64 MD (the kernel the contact forces run on)
matches the oracle to the golden parity tolerances: beads 1e-10 in position,
1e-8 in velocity; fluid 1e-10 / 1e-9.  Without the forces the two runs would
differ by far more (checked against the same run with eps = 0)."""
import numpy as np
import pytest

import cilia_gpu as cg
import simcfg
from oracle import build_from_cfg

pytestmark = pytest.mark.gpu


def periodic_diff(a, b, L):
    d = a - b
    L = np.asarray(L, dtype=float)
    return d - np.round(d / L) * L


def run(eps, steps=2):
    cfg = simcfg.swimmer_config(12, radius=2.5, n_cilia=40, rodlength=10, seed=3, ststep=0.002)
    o = build_from_cfg(cfg, seed=5, ststep=0.002)
    o.set_repelling(eps)
    s = cg.Sim(simcfg.dumps(cfg), precision=cg.MPCD_FP64, ststep=0.002, create_fluid=False)
    e = s.engine
    e.set_repelling(eps)
    p0, v0 = o.fluid()
    e.set_fluid(p0, v0)
    e.shift = o.shift
    bp, _ = s.beads()
    op, _ = o.beads()
    assert np.abs(bp - op).max() < 1e-13
    for _ in range(steps):
        rs, rg, ra, _ = o.step(record=True)
        s.next_tstep(rs, rg, ra)
    res = dict(beads=s.beads(), obeads=o.beads(), fluid=e.fluid(), ofluid=o.fluid(), contacts=o.contacts(),
               layout=e.md_layout())
    s.close()
    return res


def test_contact_forces_match_oracle():
    r = run(1000.0)
    assert r["contacts"] > 1000
    assert r["layout"]["arith"] == cg.MD_F64 and r["layout"]["cluster"] == 0
    (bp, bv), (op, ov) = r["beads"], r["obeads"]
    (p, v), (po, vo) = r["fluid"], r["ofluid"]
    errs = dict(bead_pos=np.abs(bp - op).max(), bead_vel=np.abs(bv - ov).max(),
                fluid_pos=np.abs(periodic_diff(p, po, 12)).max(), fluid_vel=np.abs(v - vo).max())
    print("repelling", r["contacts"], errs)
    assert errs["bead_pos"] < 1e-10 and errs["bead_vel"] < 1e-8, errs
    assert errs["fluid_pos"] < 1e-10 and errs["fluid_vel"] < 1e-9, errs
    # the forces matter: the run without them ends elsewhere
    r0 = run(0.0)
    assert np.abs(r0["beads"][0] - bp).max() > 1e-6
