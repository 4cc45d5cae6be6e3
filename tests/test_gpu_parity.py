"""GPU path against the reference (golden fixtures from oracle/_ref) and the
C oracle, through the C ABI.  Randomness is injected: the grid shift, the
per-cell Gamma variate and the rotation axis the reference drew, so that the
trajectories are comparable particle by particle.

Tolerances (float64 path): positions 1e-10 absolute (box edges <= 16),
velocities 1e-9 absolute, after up to 5 MPC steps / 200 MD substeps.  The
GPU uses fused multiply-adds, rsqrt and per-cell atomic sums in a different
order than the reference; the differences stay at round-off scale.
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


def ref_beads(g, tag):
    P, V = [], []
    k = 0
    while f"{tag}_obj{k}_pos" in g or k < 64:
        if f"{tag}_obj{k}_pos" in g:
            P.append(g[f"{tag}_obj{k}_pos"].reshape(-1, 3))
            V.append(g[f"{tag}_obj{k}_vel"].reshape(-1, 3))
        k += 1
    return (np.concatenate(P), np.concatenate(V)) if P else (np.zeros((0, 3)), np.zeros((0, 3)))


@pytest.mark.parametrize("case", ["fluid4", "fluid8"])
def test_fluid_matches_reference_golden(case):
    g = golden(case)
    seed, steps, ststep = g["params"]
    L = [int(x) for x in g["box"][:3]]
    e = cg.Engine(tuple(L), tstep=0.1, ststep=float(ststep), precision=cg.MPCD_FP64)
    e.set_fluid(g["step0_fluid_pos"], g["step0_fluid_vel"])
    e.shift = g["shift_0"]
    e.prepare()
    for k in range(1, int(steps) + 1):
        e.step(g[f"shift_{k}"], g[f"gamma_{k}"], g[f"axis_{k}"])
        if f"step{k}_fluid_pos" in g:
            p, v = e.fluid()
            assert np.abs(periodic_diff(p, g[f"step{k}_fluid_pos"], L)).max() < POS_TOL
            assert np.abs(v - g[f"step{k}_fluid_vel"]).max() < VEL_TOL
    obs = e.observables()
    assert abs(obs["diss_energy"] - g[f"step{int(steps)}_meta"][1]) < 1e-8 * max(1, abs(g[f"step{int(steps)}_meta"][1]))


@pytest.mark.parametrize("arith", [cg.MD_DF, cg.MD_F64, cg.MD_PAIR, cg.MD_PAIR_DF])
@pytest.mark.parametrize("case", ["clami10", "objects8"])
def test_swimmer_matches_reference_golden(case, arith):
    """MD substeps in double-float (the float64 path's default) and in float64."""
    g = golden(case)
    seed, steps, ststep = g["params"]
    text = open(f"{GOLDEN}/cases/{case}.cfg").read()
    s = cg.Sim(text, precision=cg.MPCD_FP64, ststep=float(ststep), create_fluid=False, md_arith=arith)
    e = s.engine
    assert e.md_layout()["arith"] == arith
    # geometry built by the host object model equals the reference's
    bp, bv = s.beads()
    rp, rv = ref_beads(g, "step0")
    assert bp.shape == rp.shape
    assert np.abs(bp - rp).max() < 1e-13
    e.set_fluid(g["step0_fluid_pos"], g["step0_fluid_vel"])
    e.shift = g["shift_0"]
    L = [int(x) for x in g["box"][:3]]
    for k in range(1, int(steps) + 1):
        s.next_tstep(g[f"shift_{k}"], g[f"gamma_{k}"], g[f"axis_{k}"])
    p, v = e.fluid()
    assert np.abs(periodic_diff(p, g[f"step{int(steps)}_fluid_pos"], L)).max() < POS_TOL
    assert np.abs(v - g[f"step{int(steps)}_fluid_vel"]).max() < VEL_TOL
    bp, bv = s.beads()
    rp, rv = ref_beads(g, f"step{int(steps)}")
    assert np.abs(bp - rp).max() < POS_TOL
    assert np.abs(bv - rv).max() < 1e-8
    assert abs(e.time - g[f"step{int(steps)}_meta"][0]) < 1e-12


@pytest.mark.parametrize("arith,bulk,min_tile", [(cg.MD_DF, False, 0), (cg.MD_DF, True, 0), (cg.MD_F64, False, 0),
                                                  (cg.MD_DF, False, 128), (cg.MD_DF, False, 256),
                                                  (cg.MD_PAIR, False, 0), (cg.MD_PAIR, True, 0),
                                                  (cg.MD_PAIR, False, 128), (cg.MD_PAIR, False, 256),
                                                  (cg.MD_PAIR_DF, False, 0), (cg.MD_PAIR_DF, True, 0),
                                                  (cg.MD_PAIR_DF, False, 128), (cg.MD_PAIR_DF, False, 256)])
def test_multi_tile_swimmer_matches_oracle(arith, bulk, min_tile, monkeypatch):
    """A Clami whose cilia fill many MD tiles (halos between tiles, a sphere
    centre with helper slots) against the C oracle, injected randomness, 6 MPC
    steps of 50 substeps.  bulk: the double-float kernel copies halo runs of
    two or more slots by bulk asynchronous copies (TMA) instead of per-entry
    cp.async.  min_tile: the wide tiles that large swimmers get when the
    narrow grid would not be co-resident (128 slots at four lanes per slot,
    256 at two).  MD_PAIR / MD_PAIR_DF: float64 / double-float with each
    spring pair inside a tile evaluated once and the sphere centre integrated
    from its partners' reactions."""
    if bulk:
        monkeypatch.setenv("MPCD_MD_LONG_RUN", "2")
    if min_tile:
        monkeypatch.setenv("MPCD_MD_MIN_TILE", str(min_tile))
    cfg = simcfg.swimmer_config(16, radius=4.0, n_cilia=24, rodlength=10, seed=3, ststep=0.002)
    o = build_from_cfg(cfg, seed=5, ststep=0.002)
    s = cg.Sim(simcfg.dumps(cfg), precision=cg.MPCD_FP64, ststep=0.002, create_fluid=False, md_arith=arith)
    e = s.engine
    lay = e.md_layout()
    assert lay["arith"] == arith and lay["cluster"] == 0 and lay["hmax"] > 0
    assert lay["ntiles"] > (4 if not min_tile else 2) and lay["tile"] >= min_tile
    if min_tile and arith == cg.MD_DF:
        assert lay["lanes"] == (4 if min_tile == 128 else 2)
    p0, v0 = o.fluid()
    e.set_fluid(p0, v0)
    e.shift = o.shift
    bp, _ = s.beads()
    op, _ = o.beads()
    assert np.abs(bp - op).max() < 1e-13
    L = (16, 16, 16)
    for _ in range(6):
        rs, rg, ra, _ = o.step(record=True)
        s.next_tstep(rs, rg, ra)
    bp, bv = s.beads()
    op, ov = o.beads()
    p, v = e.fluid()
    po, vo = o.fluid()
    errs = dict(bead_pos=np.abs(bp - op).max(), bead_vel=np.abs(bv - ov).max(),
                fluid_pos=np.abs(periodic_diff(p, po, L)).max(), fluid_vel=np.abs(v - vo).max())
    print("multi-tile", arith, bulk, min_tile, errs)
    assert errs["bead_pos"] < POS_TOL and errs["bead_vel"] < 1e-8, errs
    assert errs["fluid_pos"] < POS_TOL and errs["fluid_vel"] < VEL_TOL, errs
    s.close()


def _oracle_fluid(L, seed, ststep=0.002):
    o = OracleSim(L, tstep=0.1, ststep=ststep, seed=seed)
    o.init_shift()
    o.fluid_create()
    o.init_bins()
    return o


@pytest.mark.parametrize("L", [(16, 16, 16), (12, 20, 8)])
def test_fluid_matches_oracle_larger_and_ragged(L):
    """Injected run against the C oracle on non-cubic boxes."""
    o = _oracle_fluid(L, seed=21)
    p0, v0 = o.fluid()
    e = cg.Engine(L, tstep=0.1, ststep=0.002)
    e.set_fluid(p0, v0)
    e.shift = o.shift
    for _ in range(6):
        rs, rg, ra, _ = o.step(record=True)
        e.step(rs, rg, ra)
    p, v = e.fluid()
    po, vo = o.fluid()
    assert np.abs(periodic_diff(p, po, L)).max() < POS_TOL
    assert np.abs(v - vo).max() < VEL_TOL


def test_per_cell_momentum_conserved_to_roundoff():
    """The collision conserves every cell's momentum: total momentum after
    free-running steps equals the initial one to round-off."""
    o = _oracle_fluid((16, 16, 16), seed=5)
    p0, v0 = o.fluid()
    e = cg.Engine((16, 16, 16), tstep=0.1, ststep=0.002, seed=77)
    e.set_fluid(p0, v0)
    P0 = v0.sum(axis=0)
    e.run(20)
    _, v = e.fluid()
    assert np.abs(v.sum(axis=0) - P0).max() < 1e-9
    obs = e.observables()
    assert 0.95 < obs["kT"] < 1.05


def test_empty_and_sparse_cells():
    """Cells holding 0 or 1 particle: no thermostat, rotation only."""
    rng = np.random.default_rng(3)
    L = (6, 6, 6)
    n = 40  # far fewer particles than cells
    pos = rng.uniform(0, 6, (n, 3))
    vel = rng.normal(size=(n, 3))
    o = OracleSim(L, tstep=0.1, ststep=0.002, seed=9)
    o.init_shift()
    o.fluid_set(pos, vel)
    o.init_bins()
    e = cg.Engine(L, tstep=0.1, ststep=0.002)
    e.set_fluid(pos, vel)
    e.shift = o.shift
    for _ in range(4):
        rs, rg, ra, _ = o.step(record=True)
        e.step(rs, rg, ra)
    p, v = e.fluid()
    po, vo = o.fluid()
    assert np.abs(periodic_diff(p, po, L)).max() < POS_TOL
    assert np.abs(v - vo).max() < VEL_TOL


def test_injected_gamma_missing_raises():
    g = golden("fluid4")
    e = cg.Engine((4, 4, 4), tstep=0.1, ststep=0.002)
    e.set_fluid(g["step0_fluid_pos"], g["step0_fluid_vel"])
    e.shift = g["shift_0"]
    gam = np.full_like(g["gamma_1"], -1.0)
    with pytest.raises(cg.MpcdError, match="gamma"):
        e.step(g["shift_1"], gam, g["axis_1"])


def test_invalid_arguments_rejected():
    with pytest.raises(cg.MpcdError):
        cg.Engine((1, 4, 4))
    e = cg.Engine((4, 4, 4))
    with pytest.raises(cg.MpcdError):
        e.shift = [1.5, 0.0, 0.0]
    with pytest.raises(cg.MpcdError):
        cg.Sim("name = \"x\"; md_objects = ( );")  # missing root keys


def test_non_finite_input_rejected():
    e = cg.Engine((4, 4, 4))
    pos = np.zeros((2, 3))
    vel = np.zeros((2, 3))
    pos[1, 0] = np.nan
    with pytest.raises(cg.MpcdError, match="non-finite"):
        e.set_fluid(pos, vel)


@pytest.mark.parametrize("precision", [cg.MPCD_FP64, cg.MPCD_FP32])
def test_fluid_upload_download_round_trip(precision):
    """set_fluid wraps unwrapped positions into the box and splits them into
    the device layout on the device; fluid() returns them in the caller's
    order.  A rejected upload leaves the resident fluid as it was."""
    L = (6, 5, 7)
    rng = np.random.default_rng(3)
    n = 5000
    pos = rng.uniform(-20.0, 30.0, (n, 3))
    vel = rng.normal(size=(n, 3))
    e = cg.Engine(L, tstep=0.1, ststep=0.002, precision=precision)
    e.set_fluid(pos, vel)
    p, v = e.fluid()
    want = np.mod(pos, np.array(L, dtype=float))
    f64 = precision == cg.MPCD_FP64
    # float64: exact up to the wrap's rounding; float32: offsets in [0, 1) as float
    assert np.abs(periodic_diff(p, want, L)).max() < (1e-12 if f64 else 1e-7)
    assert np.all((p >= 0.0) & (p < np.array(L, dtype=float)))
    if f64:
        assert np.array_equal(v, vel)
    else:
        assert np.array_equal(v, vel.astype(np.float32).astype(np.float64))
    bad = pos.copy()
    bad[7, 2] = np.inf
    with pytest.raises(cg.MpcdError, match="non-finite"):
        e.set_fluid(bad, vel)
    p2, v2 = e.fluid()
    assert np.array_equal(p2, p) and np.array_equal(v2, v)
    # the same copies from and into page-locked caller buffers
    pin_pos, pin_vel = pos.copy(), vel.copy()
    outp, outv = np.empty_like(pos), np.empty_like(vel)
    for a in (pin_pos, pin_vel, outp, outv):
        e.pin(a)
    e.set_fluid(pin_pos, pin_vel)
    e.fluid(out=(outp, outv))
    assert np.array_equal(outp, p) and np.array_equal(outv, v)
    for a in (pin_pos, pin_vel, outp, outv):
        e.unpin(a)
    with pytest.raises(ValueError):
        e.fluid(out=(np.empty((n, 3), dtype=np.float32), outv))


def test_observables_from_cell_sums_match_particle_sums():
    """After a step the float64 engine reads its observables from the cell sums
    binned at the end of the step (fluid and moving beads, m v and m v^2 once
    each); they match the sums over the particles and beads themselves, which
    the engine takes when a setter has invalidated the binning."""
    import simcfg

    cfg = simcfg.swimmer_config(16, radius=4.0, n_cilia=12, rodlength=8, seed=3, ststep=0.002)
    s = cg.Sim(simcfg.dumps(cfg), precision=cg.MPCD_FP64, ststep=0.002, seed=4)
    e = s.engine
    e.run(3)
    a = e.observables()
    e.shift = e.shift  # the same shift: the binning is invalidated, the state unchanged
    b = e.observables()
    for k in ("kT", "fluid_T", "n", "mass", "diss_energy", "energy_fluid"):
        assert a[k] == pytest.approx(b[k], rel=1e-12, abs=1e-12), k
    assert np.abs(a["momentum"] - b["momentum"]).max() < 1e-12
    assert 16 ** 3 * 10 < a["n"] <= 16 ** 3 * 10 + s.nbeads
    s.close()


@pytest.mark.parametrize("precision", [cg.MPCD_FP64, cg.MPCD_FP32])
def test_async_observables_match_sync_and_reject_stale_tickets(precision):
    """mpcd_observables_async / mpcd_observables_result: a ticket taken after a
    step and collected several steps later (out of order) holds what
    mpcd_observables returned right after that step, globalt included; tickets
    never issued or older than the ring are rejected, the newest stay valid."""
    import simcfg

    cfg = simcfg.swimmer_config(16, radius=4.0, n_cilia=12, rodlength=8, seed=3, ststep=0.002)
    s = cg.Sim(simcfg.dumps(cfg), precision=precision, ststep=0.002, seed=4)
    e = s.engine
    tickets, sync = [], []
    for _ in range(5):
        e.step()
        tickets.append(e.observables_async())
        sync.append(e.observables())
    for t, want in reversed(list(zip(tickets, sync))):
        got = e.observables_result(t)
        for k in ("kT", "fluid_T", "n", "mass", "diss_energy", "energy_fluid", "globalt"):
            assert got[k] == pytest.approx(want[k], rel=1e-12, abs=1e-14), k
        assert np.abs(got["momentum"] - want["momentum"]).max() < 1e-14
    assert len({o["globalt"] for o in sync}) == len(sync)
    first = tickets[0]
    latest = [e.observables_async() for _ in range(cg.OBS_RING)]
    with pytest.raises(cg.MpcdError, match="overwritten"):
        e.observables_result(first)
    with pytest.raises(cg.MpcdError, match="not issued"):
        e.observables_result(latest[-1] + 1)
    with pytest.raises(cg.MpcdError, match="not issued"):
        e.observables_result(-1)
    a, b = e.observables_result(latest[0]), e.observables_result(latest[-1])
    # the same state each time; the float32 path's sums are atomic additions,
    # so they agree to the order of those additions
    c = e.observables()
    assert a["kT"] == pytest.approx(c["kT"], rel=1e-12) and b["kT"] == pytest.approx(c["kT"], rel=1e-12)
    s.close()


def test_unstable_md_step_reports_error_without_fault():
    """A too-large MD step lets the beads diverge; the kernels report it."""
    import simcfg

    cfg = simcfg.plain_fluid(12, name="unstable")
    cfg["ststep"] = 0.02
    cfg["md_objects"] = (simcfg.fibonacci_clami(6, radius=3.5, center=(6, 6, 6), rodlength=6,
                                                springconstant=20000.0, seed=1),)
    for prec in (cg.MPCD_FP64, cg.MPCD_FP32):
        s = cg.Sim(simcfg.dumps(cfg), precision=prec, seed=2)
        with pytest.raises(cg.MpcdError, match="non-finite"):
            for _ in range(40):
                s.next_tstep()
            s.engine.sync()
        s.close()
