"""Split-precision path (int cell + float32 offset, float32 velocities and
cell sums; MD in double-float by default, or split-precision springs) against
the float64 path and the reference fixtures.  Stated errors: positions 2e-4 and velocities 2e-4
absolute after 4 MPC steps of identical injected randomness; kT within 1 %
and total momentum per particle below 1e-5 over free-running steps."""
import numpy as np
import pytest

import cilia_gpu as cg
from conftest import GOLDEN, golden
from oracle import OracleSim

pytestmark = pytest.mark.gpu


def periodic_diff(a, b, L):
    d = a - b
    L = np.asarray(L, dtype=float)
    return d - np.round(d / L) * L


def test_fp32_fluid_tracks_reference_golden():
    g = golden("fluid8")
    L = (8, 8, 8)
    e = cg.Engine(L, tstep=0.1, ststep=0.002, precision=cg.MPCD_FP32)
    e.set_fluid(g["step0_fluid_pos"], g["step0_fluid_vel"])
    e.shift = g["shift_0"]
    for k in range(1, 4):
        e.step(g[f"shift_{k}"], g[f"gamma_{k}"], g[f"axis_{k}"])
    p, v = e.fluid()
    # a particle within float32 rounding of a cell face may bin differently: allow a tiny fraction
    dp = np.abs(periodic_diff(p, g["step3_fluid_pos"], L)).max(axis=1)
    dv = np.abs(v - g["step3_fluid_vel"]).max(axis=1)
    assert np.mean(dp < 2e-4) > 0.999
    assert np.mean(dv < 2e-4) > 0.995


@pytest.mark.parametrize("arith", [cg.MD_AUTO, cg.MD_DF, cg.MD_SPLIT, cg.MD_FLOAT, cg.MD_PAIR, cg.MD_PAIR_DF])
def test_fp32_swimmer_tracks_reference_golden(arith):
    """MD in split arithmetic on the double-float kernel's grid layout (the
    default of the float32 path), in double-float, in split arithmetic on
    one thread-block cluster (the replica batch's MD), and in float64 on the
    pair kernel, beside the float32 fluid."""
    g = golden("clami10")
    text = open(f"{GOLDEN}/cases/clami10.cfg").read()
    s = cg.Sim(text, precision=cg.MPCD_FP32, ststep=0.002, create_fluid=False, md_arith=arith)
    e = s.engine
    assert e.md_layout()["arith"] == (cg.MD_FLOAT if arith == cg.MD_AUTO else arith)
    e.set_fluid(g["step0_fluid_pos"], g["step0_fluid_vel"])
    e.shift = g["shift_0"]
    for k in range(1, 5):
        s.next_tstep(g[f"shift_{k}"], g[f"gamma_{k}"], g[f"axis_{k}"])
    bp, bv = s.beads()
    P = [g[f"step4_obj{k}_pos"].reshape(-1, 3) for k in range(64) if f"step4_obj{k}_pos" in g]
    rp = np.concatenate(P)
    assert np.abs(bp - rp).max() < 1e-3


def test_fp32_conservation_and_temperature():
    o = OracleSim((24, 24, 24), tstep=0.1, ststep=0.002, seed=8)
    o.init_shift()
    o.fluid_create()
    p0, v0 = o.fluid()
    e = cg.Engine((24, 24, 24), tstep=0.1, ststep=0.002, precision=cg.MPCD_FP32, seed=4)
    e.set_fluid(p0, v0)
    e.run(60)
    obs = e.observables()
    assert abs(obs["kT"] - 1.0) < 0.01
    assert np.abs(obs["momentum"]).max() < 1e-5
