"""Parity at the benchmark sizes, through the C ABI, with the randomness
injected from the C oracle (grid shift, per-cell Gamma variate and rotation
axis of every step), so that trajectories compare particle by particle.

  plain32   : the 32^3 periodic fluid of the plain-fluid benchmark (327,680
              particles), 3 MPC steps.
  swimmer64 : the 64^3 box with the radius-8 Clami of 100 Fibonacci-lattice
              cilia (3 x 15 beads, 5,143 beads, 50 MD substeps per step) of
              the single-swimmer benchmark, 2 MPC steps, MD in double-float
              (the float64 path's default) and in IEEE float64.
  fluid72   : a 72^3 box (3.73 M particles) with a small swimmer: the fluid
              pass beside the MD launch runs at its cap of short-lived CTAs
              with more than one round of particles per thread.

These sizes take the kernels through paths the small golden cases do not:
32-bit particle indices over many CTAs, the short-lived CTA cap, MD tile
counts near co-residency, the sort every 50 steps (plain32 is run past it).

Tolerances as the golden parity tests: float64 positions 1e-10 absolute,
velocities 1e-9 (beads 1e-8); split precision 2e-4 for 99.9 % of the
particles.  Also here: the product's Fluid::create (cilia_sim_create with
create_fluid) against the reference's own initial state, bitwise.
"""
import numpy as np
import pytest

import cilia_gpu as cg
import simcfg
from conftest import GOLDEN, golden
from oracle import OracleSim, build_from_cfg

pytestmark = pytest.mark.gpu

POS_TOL = 1e-10
VEL_TOL = 1e-9


def periodic_diff(a, b, L):
    d = a - b
    L = np.asarray(L, dtype=float)
    return d - np.round(d / L) * L


@pytest.mark.parametrize("precision", [cg.MPCD_FP64, cg.MPCD_FP32])
def test_plain32_matches_oracle(precision):
    L = (32, 32, 32)
    o = OracleSim(L, tstep=0.1, ststep=0.002, seed=31)
    o.init_shift()
    o.fluid_create()
    o.init_bins()
    p0, v0 = o.fluid()
    assert p0.shape[0] == 327680
    # sort every 2 steps: the run crosses a counting-sort reorder
    e = cg.Engine(L, tstep=0.1, ststep=0.002, precision=precision, sort_interval=2)
    e.set_fluid(p0, v0)
    e.shift = o.shift
    for _ in range(3):
        rs, rg, ra, _ = o.step(record=True)
        e.step(rs, rg, ra)
    p, v = e.fluid()
    po, vo = o.fluid()
    dp = np.abs(periodic_diff(p, po, L)).max(axis=1)
    dv = np.abs(v - vo).max(axis=1)
    if precision == cg.MPCD_FP64:
        assert dp.max() < POS_TOL and dv.max() < VEL_TOL, (dp.max(), dv.max())
        obs = e.observables()
        # a difference of two sums of ~5e5 each, added in another order
        assert abs(obs["diss_energy"] - o.diss_energy()) < 1e-8 * max(1.0, abs(o.diss_energy())) + 1e-6
    else:
        assert np.mean(dp < 2e-4) > 0.999 and np.mean(dv < 2e-4) > 0.999, (np.sort(dp)[-3:], np.sort(dv)[-3:])


@pytest.mark.parametrize("arith", [cg.MD_DF, cg.MD_F64, cg.MD_PAIR, cg.MD_PAIR_DF])
def test_swimmer64_matches_oracle(arith):
    cfg = simcfg.baseline_config("swimmer64", seed=3)
    o = build_from_cfg(cfg, seed=5, ststep=0.002)
    s = cg.Sim(simcfg.dumps(cfg), precision=cg.MPCD_FP64, ststep=0.002, create_fluid=False, md_arith=arith)
    e = s.engine
    lay = e.md_layout()
    assert lay["arith"] == arith
    assert s.nbeads == o.bead_count() == 643 + 100 * 45
    if arith in (cg.MD_PAIR, cg.MD_PAIR_DF):
        # the sphere centre's 642 radial springs are dropped: its force is the
        # negated sum of the surface beads' reactions
        d = cg.Sim(simcfg.dumps(cfg), precision=cg.MPCD_FP64, ststep=0.002, create_fluid=False, md_arith=cg.MD_DF)
        assert lay["nsprings"] == d.engine.md_layout()["nsprings"] - 642
        d.close()
    bp, _ = s.beads()
    op, _ = o.beads()
    assert np.abs(bp - op).max() < 1e-13
    p0, v0 = o.fluid()
    assert p0.shape[0] == 64 ** 3 * 10
    e.set_fluid(p0, v0)
    e.shift = o.shift
    for _ in range(2):
        rs, rg, ra, _ = o.step(record=True)
        s.next_tstep(rs, rg, ra)
    L = (64, 64, 64)
    p, v = e.fluid()
    po, vo = o.fluid()
    bp, bv = s.beads()
    op, ov = o.beads()
    errs = dict(fluid_pos=np.abs(periodic_diff(p, po, L)).max(), fluid_vel=np.abs(v - vo).max(),
                bead_pos=np.abs(bp - op).max(), bead_vel=np.abs(bv - ov).max())
    print("swimmer64", arith, lay, errs)
    assert errs["fluid_pos"] < POS_TOL and errs["fluid_vel"] < VEL_TOL, errs
    assert errs["bead_pos"] < POS_TOL and errs["bead_vel"] < 1e-8, errs
    s.close()


def test_fluid72_multi_round_fluid_pass_matches_oracle():
    cfg = simcfg.swimmer_config(72, radius=4.0, n_cilia=6, rodlength=8, seed=2, ststep=0.002)
    o = build_from_cfg(cfg, seed=9, ststep=0.002)
    s = cg.Sim(simcfg.dumps(cfg), precision=cg.MPCD_FP64, ststep=0.002, create_fluid=False)
    e = s.engine
    p0, v0 = o.fluid()
    assert p0.shape[0] == 72 ** 3 * 10 > 10240 * 256  # beyond one round of the capped grid
    e.set_fluid(p0, v0)
    e.shift = o.shift
    for _ in range(2):
        rs, rg, ra, _ = o.step(record=True)
        s.next_tstep(rs, rg, ra)
    L = (72, 72, 72)
    p, v = e.fluid()
    po, vo = o.fluid()
    bp, _ = s.beads()
    op, _ = o.beads()
    assert np.abs(periodic_diff(p, po, L)).max() < POS_TOL
    assert np.abs(v - vo).max() < VEL_TOL
    assert np.abs(bp - op).max() < POS_TOL
    s.close()


@pytest.mark.parametrize("case", ["fluid4", "fluid8", "clami10", "objects8"])
def test_create_fluid_matches_reference_initial_state(case):
    """Simulation's constructor with the fluid created (Fluid::create,
    src/libcilia/fluid.cpp:55-98, after MPCD's grid shift and the md_objects'
    own draws from the same generator) gives the reference's initial grid
    shift and fluid positions bit for bit, and its velocities to 1e-14: the
    reference is compiled with -ffast-math, so its Box-Muller transform and
    the mean-velocity subtraction may round differently in the last bit."""
    g = golden(case)
    seed = int(g["params"][0])
    text = open(f"{GOLDEN}/cases/{case}.cfg").read()
    s = cg.Sim(text, precision=cg.MPCD_FP64, ststep=float(g["params"][2]), seed=seed, create_fluid=True)
    e = s.engine
    assert np.array_equal(e.shift, g["shift_0"])
    p, v = e.fluid()
    assert p.shape == g["step0_fluid_pos"].shape
    assert np.array_equal(p, g["step0_fluid_pos"])
    assert np.abs(v - g["step0_fluid_vel"]).max() < 1e-14
    s.close()
