"""Replica batch (include/mpcd_batch.h): many boxes advanced together.

A replica's random numbers are keyed by its own seed, step counter and cell
indices, exactly as the single-box split-precision engine keys them, so a
replica must follow the trajectory of the same box run alone in the engine,
and must not depend on which other replicas share the batch.  What may
differ is the order of float additions into the cell sums (atomics) and the
MD layout (slots per CTA), hence the split-precision tolerances of
test_gpu_fp32: 99.9 % of the fluid particles within 1e-4 in position and
velocity after a few steps, beads within 1e-3.
"""
import numpy as np
import pytest

import cilia_gpu as cg
import simcfg

pytestmark = pytest.mark.gpu


def periodic_diff(a, b, L):
    d = a - b
    return d - np.round(d / float(L)) * float(L)


def make_batch(specs, **kw):
    nf = sum(10 * s["L"] ** 3 for s in specs)
    nc = sum(s["L"] ** 3 for s in specs)
    nb = sum(643 + 3 * s["n_cilia"] * s["rodlength"] for s in specs)
    args = dict(max_replicas=max(len(specs), 1) + 2, max_particles=nf + 8192 * len(specs),
                max_cells=nc + 2048 * len(specs), max_slots=2 * nb + 1024 * len(specs), max_springs=14 * nb,
                max_halo=6 * nb + 4096, max_cilia=sum(s["n_cilia"] for s in specs) + 1,
                max_bonds=sum(s["n_cilia"] * s["rodlength"] for s in specs) + 1)
    args.update(kw)
    return cg.Batch(**args)


def swimmer_sim(spec):
    cfg = simcfg.swimmer_config(spec["L"], radius=spec["radius"], n_cilia=spec["n_cilia"],
                                rodlength=spec["rodlength"], seed=spec["seed"])
    return cg.Sim(simcfg.dumps(cfg), precision=cg.MPCD_FP32, ststep=0.002, seed=spec["seed"])


def fluid_close(p1, v1, p2, v2, L, tol=1e-4, frac=0.999):
    dp = np.abs(periodic_diff(p1, p2, L)).max(axis=1)
    dv = np.abs(v1 - v2).max(axis=1)
    return np.mean(dp < tol) > frac and np.mean(dv < tol) > frac, (np.sort(dp)[-3:], np.sort(dv)[-3:])


def test_plain_replica_matches_engine():
    L, n, seed = 16, 16 ** 3 * 10, 21
    rng = np.random.default_rng(3)
    pos = rng.uniform(0, L, (n, 3))
    vel = rng.normal(size=(n, 3))
    vel -= vel.mean(axis=0)
    e = cg.Engine(L, tstep=0.1, ststep=0.002, precision=cg.MPCD_FP32, seed=seed)
    e.set_fluid(pos, vel)
    b = make_batch([dict(L=L, n_cilia=0, rodlength=10)])
    r = b.add(L, seed=seed)
    b.set_fluid(r, pos, vel)
    b.set_shift(r, e.shift)
    b.admit(r)
    b.set_steps(r, 5)
    e.run(5)
    b.run(5)
    pe, ve = e.fluid()
    pb, vb = b.fluid(r, n)
    ok, worst = fluid_close(pe, ve, pb, vb, L)
    assert ok, worst
    oe, ob = e.observables(), b.observables(r)
    assert abs(oe["kT"] - ob["kT"]) < 1e-4
    assert abs(oe["diss_energy"] - ob["diss_energy"]) <= 1e-3 * max(1.0, abs(oe["diss_energy"]))
    assert b.status(r)["steps"] == 5 and abs(b.status(r)["globalt"] - e.time) < 1e-12


def test_swimmer_replica_matches_engine():
    spec = dict(L=16, radius=2.0, n_cilia=6, rodlength=10, seed=7)
    s = swimmer_sim(spec)
    b = make_batch([spec])
    r = b.add_engine(s.engine)
    b.admit(r)
    b.set_steps(r, 4)
    s.engine.run(4)
    b.run(4)
    nb = s.nbeads
    bp_e, bv_e = s.beads()
    bp_b, bv_b = b.beads(r, nb)
    assert np.abs(bp_e - bp_b).max() < 1e-3
    assert np.abs(bv_e - bv_b).max() < 1e-2
    n = 10 * spec["L"] ** 3
    pe, ve = s.engine.fluid()
    pb, vb = b.fluid(r, n)
    ok, worst = fluid_close(pe, ve, pb, vb, spec["L"])
    assert ok, worst


def test_replica_same_alone_and_in_mix():
    specs = simcfg.ensemble_specs(6, seed=5, edges=(16, 24), max_cilia=12, rodlengths=(10, 12))
    target = dict(L=16, radius=2.0, n_cilia=5, rodlength=10, seed=99)
    sims = [swimmer_sim(x) for x in specs + [target]]
    alone = make_batch([target])
    mix = make_batch(specs + [target])
    ra = alone.add_engine(sims[-1].engine)
    alone.admit(ra)
    ids = []
    for sim in sims:  # the target is admitted last, between the others' ranges
        k = mix.add_engine(sim.engine)
        mix.admit(k)
        ids.append(k)
    rm = ids[-1]
    for k in ids:
        mix.set_steps(k, 6)
    alone.set_steps(ra, 6)
    alone.run(6)
    mix.run(6)
    nb = sims[-1].nbeads
    pa, va = alone.beads(ra, nb)
    pm, vm = mix.beads(rm, nb)
    assert np.abs(pa - pm).max() < 1e-3
    n = 10 * 16 ** 3
    fa = alone.fluid(ra, n)
    fm = mix.fluid(rm, n)
    ok, worst = fluid_close(fa[0], fa[1], fm[0], fm[1], 16)
    assert ok, worst
    for k in ids:
        st = mix.status(k)
        assert st["steps"] == 6 and st["err"] == 0


def test_step_budgets_and_conservation():
    specs = [dict(L=16, n_cilia=0, rodlength=10), dict(L=24, n_cilia=0, rodlength=10)]
    b = make_batch(specs)
    rng = np.random.default_rng(1)
    rs = []
    for k, sp in enumerate(specs):
        L = sp["L"]
        n = 10 * L ** 3
        pos = rng.uniform(0, L, (n, 3))
        vel = rng.normal(size=(n, 3))
        vel -= vel.mean(axis=0)
        r = b.add(L, seed=100 + k)
        b.set_fluid(r, pos, vel)
        b.admit(r)
        rs.append(r)
    b.set_steps(rs[0], 10)
    b.set_steps(rs[1], 40)
    b.run(60)
    assert b.status(rs[0])["steps"] == 10 and b.status(rs[0])["steps_left"] == 0
    assert b.status(rs[1])["steps"] == 40
    for r in rs:
        o = b.observables(r)
        assert np.abs(o["momentum"]).max() < 1e-5
        assert abs(o["kT"] - 1.0) < 0.03


def test_admit_remove_and_capacity():
    b = make_batch([dict(L=16, n_cilia=0, rodlength=10)], max_replicas=3)
    rng = np.random.default_rng(2)
    n = 10 * 16 ** 3
    pos = rng.uniform(0, 16, (n, 3))
    vel = rng.normal(size=(n, 3))
    r1 = b.add(16, seed=1)
    b.set_fluid(r1, pos, vel)
    b.admit(r1)
    r2 = b.add(16, seed=2)
    b.set_fluid(r2, pos, vel)
    assert not b.try_admit(r2)  # the particle capacity holds one 16^3 box
    b.set_steps(r1, 3)
    b.run(3)
    b.remove(r1)
    assert b.resident == 0
    b.admit(r2)  # reuses the freed ranges
    b.set_steps(r2, 3)
    b.run(3)
    assert b.status(r2)["steps"] == 3
    o = b.observables(r2)
    assert abs(o["kT"] - 1.0) < 0.05


def test_autotune_picks_a_valid_configuration():
    specs = simcfg.ensemble_specs(4, seed=2, edges=(16, 24), max_cilia=8, rodlengths=(10, 11))
    sims = [swimmer_sim(x) for x in specs]
    b = make_batch(specs)
    ids = []
    for s in sims:
        k = b.add_engine(s.engine)
        b.admit(k)
        b.set_steps(k, 10 ** 6)
        ids.append(k)
    t = b.autotune(trial_steps=20)
    assert t["fluid_threads"] in (256, 512) and t["sort_interval"] in (10, 25, 50, 100)
    b.run(10)
    for k in ids:
        st = b.status(k)
        assert st["err"] == 0 and st["steps"] > 100
        o = b.observables(k)
        assert 0.8 < o["kT"] < 1.3


def test_md_relayout_continues_the_trajectory():
    spec = dict(L=16, radius=2.0, n_cilia=8, rodlength=10, seed=17)
    s = swimmer_sim(spec)
    b1, b2 = make_batch([spec]), make_batch([spec])
    r1, r2 = b1.add_engine(s.engine), b2.add_engine(s.engine)
    b1.admit(r1)
    b2.admit(r2)
    for b, r in ((b1, r1), (b2, r2)):
        b.set_steps(r, 6)
        b.run(3)
    b2.set_md_layout(1, 512)
    assert b2.md_layout() == (1, 512)
    b1.run(3)
    b2.run(3)
    nb = s.nbeads
    p1, v1 = b1.beads(r1, nb)
    p2, v2 = b2.beads(r2, nb)
    assert np.abs(p1 - p2).max() < 1e-3
    assert b2.status(r2)["steps"] == 6 and b2.status(r2)["err"] == 0


def test_shared_memory_staged_fluid_pass_matches_the_direct_pass():
    """The fluid pass staged by bulk copies (tuning fluid_threads = 0) gives the
    direct pass's trajectory (same arithmetic; only atomics order differs)."""
    specs = [dict(L=16, n_cilia=0, rodlength=10), dict(L=24, n_cilia=0, rodlength=10)]
    rng = np.random.default_rng(4)
    data = []
    for sp in specs:
        n = 10 * sp["L"] ** 3
        pos = rng.uniform(0, sp["L"], (n, 3))
        vel = rng.normal(size=(n, 3))
        data.append((pos, vel - vel.mean(axis=0)))
    out = []
    for threads in (256, 0):
        b = make_batch(specs)
        b.set_tuning(fluid_threads=threads, fluid_blocks=0)
        rs = []
        for k, sp in enumerate(specs):
            r = b.add(sp["L"], seed=40 + k)
            b.set_fluid(r, *data[k])
            b.admit(r)
            b.set_steps(r, 5)
            rs.append(r)
        b.run(5)
        out.append([b.fluid(r, 10 * sp["L"] ** 3) for r, sp in zip(rs, specs)])
        for r in rs:
            assert b.status(r)["err"] == 0 and b.status(r)["steps"] == 5
        b.close()
    for (p1, v1), (p2, v2), sp in zip(out[0], out[1], specs):
        ok, worst = fluid_close(p1, v1, p2, v2, sp["L"])
        assert ok, worst


def ref_bead_pos(g, tag):
    P = [g[f"{tag}_obj{k}_pos"].reshape(-1, 3) for k in range(64) if f"{tag}_obj{k}_pos" in g]
    return np.concatenate(P)


def test_replica_with_injected_randomness_tracks_reference_fluid():
    """One replica of the batch run on the reference's recorded randomness
    (mpcd_batch_step_inject) against the reference's own trajectory
    (tests/golden/fluid8.npz), beside an uninjected replica that keeps
    running on its generator: split-precision tolerances of test_gpu_fp32."""
    from conftest import golden

    g = golden("fluid8")
    L = 8
    b = make_batch([dict(L=L, n_cilia=0, rodlength=10), dict(L=16, n_cilia=0, rodlength=10)])
    other = b.add(16, seed=5)
    rng = np.random.default_rng(2)
    po = rng.uniform(0, 16, (16 ** 3 * 10, 3))
    vo = rng.normal(size=po.shape)
    b.set_fluid(other, po, vo)
    b.admit(other)
    b.set_steps(other, 10)
    r = b.add(L, seed=1)
    b.set_fluid(r, g["step0_fluid_pos"], g["step0_fluid_vel"])
    b.set_shift(r, g["shift_0"])
    b.admit(r)
    b.set_steps(r, 3)
    for k in range(1, 4):
        b.step_inject(r, g[f"shift_{k}"], g[f"gamma_{k}"], g[f"axis_{k}"])
        assert np.array_equal(b.shift(r), g[f"shift_{k}"])
    p, v = b.fluid(r, g["step3_fluid_pos"].shape[0])
    dp = np.abs(periodic_diff(p, g["step3_fluid_pos"], L)).max(axis=1)
    dv = np.abs(v - g["step3_fluid_vel"]).max(axis=1)
    assert np.mean(dp < 2e-4) > 0.999, np.sort(dp)[-3:]
    assert np.mean(dv < 2e-4) > 0.995, np.sort(dv)[-3:]
    assert b.status(r)["steps"] == 3 and b.status(other)["steps"] == 3
    # a missing Gamma variate for a thermostatted cell is reported
    b.set_steps(r, 1)
    with pytest.raises(cg.MpcdError, match="gamma"):
        b.step_inject(r, g["shift_1"], np.full_like(g["gamma_1"], -1.0), g["axis_1"])
    b.close()


def test_swimmer_replica_with_injected_randomness_tracks_reference():
    """A Clami replica (the batch's split-arithmetic cluster MD) on the
    reference's recorded randomness against its trajectory
    (tests/golden/clami10.npz): beads within 1e-3 after 4 MPC steps of 50
    substeps, as the single-box split-arithmetic MD."""
    from conftest import GOLDEN, golden

    g = golden("clami10")
    text = open(f"{GOLDEN}/cases/clami10.cfg").read()
    b = make_batch([dict(L=10, n_cilia=4, rodlength=6)])
    r = b.add_cfg(text, seed=3, ststep=0.002, create_fluid=False)
    b.set_fluid(r, g["step0_fluid_pos"], g["step0_fluid_vel"])
    b.set_shift(r, g["shift_0"])
    b.admit(r)
    b.set_steps(r, 4)
    for k in range(1, 5):
        b.step_inject(r, g[f"shift_{k}"], g[f"gamma_{k}"], g[f"axis_{k}"])
    rp = ref_bead_pos(g, "step4")
    bp, _ = b.beads(r, rp.shape[0])
    assert np.abs(bp - rp).max() < 1e-3, np.abs(bp - rp).max()
    p, v = b.fluid(r, g["step4_fluid_pos"].shape[0])
    dp = np.abs(periodic_diff(p, g["step4_fluid_pos"], 10)).max(axis=1)
    assert np.mean(dp < 2e-4) > 0.999, np.sort(dp)[-3:]
    b.close()
