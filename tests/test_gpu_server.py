"""Continuous batching server (include/mpcd_server.h).

Requests are sim.cfg texts with a step count and a seed.  A request's
random numbers are keyed by its own seed and step counter, so its result is
the same whether it ran alone or while other requests were admitted,
running and retired around it, up to the order of float additions into its
cell sums.  That order is not reproducible even between two runs alone, and
the dynamics amplify it (a particle within rounding of a cell face changes
collision partners), so:
  - over a short run (8 steps) the alone and mixed results agree: beads
    within 1e-3, 99.9 % of the fluid positions within 1e-4, kT within 1e-4,
    and the share of fluid velocities off by more than 1e-4 (particles in the
    swimmer's cells, which feel its float-rounded bead velocities) is at most
    2x (+0.5 %) that share between two runs alone;
  - over a longer run (40 steps) the difference between the alone and the
    mixed result is of the size of the differences among runs alone.  Those
    scatter widely (maximum bead deviations between two runs alone measured
    from 0.005 to 0.09 after 40 steps), so the reference is the largest of
    the three pairwise differences among three runs alone, and the mixed
    result's difference is the median over those three runs; it must stay
    within 3x (+1e-3) of the reference, both in the largest and in the RMS
    bead deviation; kT agrees with the runs alone within 3x their spread
    (at least 2e-3).
"""
import time

import numpy as np
import pytest

import cilia_gpu as cg
import simcfg

pytestmark = pytest.mark.gpu


def request_cfg(L, n_cilia, rodlength=10, seed=0):
    return simcfg.dumps(simcfg.swimmer_config(L, radius=L / 8.0, n_cilia=n_cilia, rodlength=rodlength, seed=seed))


def capacity(n, L=24, n_cilia=8, rodlength=10, **kw):
    nb = 643 + 3 * n_cilia * rodlength
    c = dict(max_replicas=n + 2, max_particles=n * (10 * L ** 3 + 8192), max_cells=n * (L ** 3 + 2048),
             max_slots=n * (2 * nb + 1024), max_springs=n * 14 * nb, max_halo=n * (6 * nb + 4096),
             max_cilia=n * n_cilia + 1, max_bonds=n * n_cilia * rodlength + 1)
    c.update(kw)
    return c


def periodic_diff(a, b, L):
    d = a - b
    return d - np.round(d / float(L)) * float(L)


def test_requests_complete_with_latency_stats():
    srv = cg.Server(chunk_steps=10, **capacity(6))
    ids = []
    for k, (L, nc, steps) in enumerate([(16, 0, 30), (24, 6, 20), (16, 4, 50), (24, 0, 10), (16, 8, 40)]):
        ids.append((srv.submit(request_cfg(L, nc, seed=k), steps, seed=100 + k), steps))
    srv.drain(300)
    for rid, steps in ids:
        info = srv.wait(rid, 10)
        assert info["state"] == cg.REQ_DONE and info["steps"] == steps and info["err"] == 0
        assert info["t_submit"] <= info["t_admit"] <= info["t_done"]
        assert 0.8 < info["obs"]["kT"] < 1.3
    st = srv.stats()
    assert st["completed"] == 5 and st["failed"] == 0
    assert 0 < st["p50_s"] <= st["p99_s"] <= st["max_s"]
    assert st["throughput"] > 0 and st["gpu_launches"] > 0
    srv.close()


def run_alone(target, steps, seed):
    srv = cg.Server(chunk_steps=10, keep_fluid=True, **capacity(2))
    rid = srv.submit(target, steps, seed=seed)
    info = srv.wait(rid, 300)
    beads = srv.result_beads(rid, info["nbeads"])
    fluid = srv.result_fluid(rid, info["nfluid"])
    srv.close()
    return info, beads, fluid


def run_in_mix(target, steps, seed):
    mix = cg.Server(chunk_steps=7, keep_fluid=True, **capacity(6))
    for k, (L, nc, st) in enumerate([(24, 6, 60), (16, 0, 15), (16, 8, 90)]):
        mix.submit(request_cfg(L, nc, seed=10 + k), st, seed=500 + k)
    rid = mix.submit(target, steps, seed=seed)  # joins a batch already running
    mix.submit(request_cfg(24, 2, seed=20), 30, seed=600)
    info = mix.wait(rid, 300)
    beads = mix.result_beads(rid, info["nbeads"])
    fluid = mix.result_fluid(rid, info["nfluid"])
    mix.drain(300)
    peak = mix.stats()["peak_resident"]
    mix.close()
    return info, beads, fluid, peak


def test_result_same_alone_and_in_the_mix():
    target = request_cfg(16, 5, seed=3)
    ia, (pa, _), fa = run_alone(target, 8, 77)
    _, _, fb = run_alone(target, 8, 77)
    im, (pm, _), fm, peak = run_in_mix(target, 8, 77)
    assert im["steps"] == ia["steps"] == 8 and peak >= 2
    assert np.abs(pa - pm).max() < 1e-3
    dp = np.abs(periodic_diff(fa[0], fm[0], 16)).max(axis=1)
    assert np.mean(dp < 1e-4) > 0.999
    off_mix = np.mean(np.abs(fa[1] - fm[1]).max(axis=1) > 1e-4)
    off_rep = np.mean(np.abs(fa[1] - fb[1]).max(axis=1) > 1e-4)
    assert off_mix <= 2 * off_rep + 0.005, (off_mix, off_rep)
    assert abs(ia["obs"]["kT"] - im["obs"]["kT"]) < 1e-4


def test_long_run_mix_within_the_run_to_run_spread():
    target = request_cfg(16, 5, seed=3)
    alone = [run_alone(target, 40, 77) for _ in range(3)]
    im, (pm, _), _, _ = run_in_mix(target, 40, 77)
    pos = [b[0] for _, b, _ in alone]

    def dev(a, b):
        d = np.abs(a - b)
        return d.max(), float(np.sqrt((d ** 2).mean()))

    ref = [dev(pos[i], pos[j]) for i, j in ((0, 1), (0, 2), (1, 2))]
    mix = [dev(p, pm) for p in pos]
    ref_max, ref_rms = max(r[0] for r in ref), max(r[1] for r in ref)
    mix_max, mix_rms = float(np.median([m[0] for m in mix])), float(np.median([m[1] for m in mix]))
    assert mix_max < 3 * ref_max + 1e-3, (mix_max, ref_max, ref, mix)
    assert mix_rms < 3 * ref_rms + 1e-3, (mix_rms, ref_rms, ref, mix)
    # kT of diverged trajectories of a 16^3 box differs by its thermal spread
    # (relative 1/sqrt(3N/2), about 0.005 here): against the runs alone
    kts = [info["obs"]["kT"] for info, _, _ in alone]
    kt_spread = max(abs(a - b) for a in kts for b in kts)
    assert abs(im["obs"]["kT"] - float(np.median(kts))) < 3 * max(kt_spread, 2e-3), (im["obs"]["kT"], kts)


def test_admission_respects_the_budget():
    probe = cg.Batch.for_specs([dict(L=16, n_cilia=4, rodlength=10)])
    r = probe.add_cfg(request_cfg(16, 4), seed=1)
    fp = probe.footprint(r)
    probe.close()
    srv = cg.Server(chunk_steps=10, budget_bytes=int(2.5 * fp), **capacity(6, L=16, n_cilia=4))
    ids = [srv.submit(request_cfg(16, 4, seed=k), 20, seed=k + 1) for k in range(5)]
    srv.drain(300)
    st = srv.stats()
    assert st["completed"] == 5
    assert st["peak_resident"] <= 2 and st["peak_resident_bytes"] <= 2.5 * fp
    for rid in ids:
        assert srv.info(rid)["state"] == cg.REQ_DONE
    srv.close()


def test_bad_request_fails_alone():
    srv = cg.Server(chunk_steps=10, **capacity(3, L=16))
    bad = srv.submit("sizex = ;", 10, seed=1)
    good = srv.submit(request_cfg(16, 2), 10, seed=2)
    with pytest.raises(cg.MpcdError):
        srv.wait(bad, 60)
    assert srv.info(bad)["state"] == cg.REQ_FAILED
    assert srv.wait(good, 300)["state"] == cg.REQ_DONE
    srv.close()


def test_preempted_request_resumes_like_an_uninterrupted_run():
    """A request pre-empted mid-run (mpcd_server_preempt: its state read back
    to the host, its device ranges freed) and admitted again continues its
    own random sequence: after 8 steps it agrees with the same request run
    alone without interruption within the short-run tolerances above (beads
    1e-3, 99.9 % of fluid positions 1e-4, kT 1e-4), ran all its steps and
    reports the pre-emption."""
    target = request_cfg(16, 5, seed=3)
    steps = 8
    ia, (pa, _), fa = run_alone(target, steps, 77)
    srv = cg.Server(chunk_steps=2, keep_fluid=True, **capacity(3))
    rid = srv.submit(target, steps, seed=77)
    t0 = time.time()
    while srv.info(rid)["state"] != cg.REQ_RESIDENT and time.time() - t0 < 60:
        time.sleep(0.002)
    assert srv.preempt(rid)
    info = srv.wait(rid, 300)
    pm, _ = srv.result_beads(rid, info["nbeads"])
    fm = srv.result_fluid(rid, info["nfluid"])
    assert srv.stats()["preemptions"] >= 1
    srv.close()
    assert info["state"] == cg.REQ_DONE and info["steps"] == steps and info["preemptions"] >= 1
    assert np.abs(pa - pm).max() < 1e-3
    dp = np.abs(periodic_diff(fa[0], fm[0], 16)).max(axis=1)
    assert np.mean(dp < 1e-4) > 0.999
    assert abs(ia["obs"]["kT"] - info["obs"]["kT"]) < 1e-4


def test_preemption_policy_lets_a_short_request_pass_a_long_one():
    """With room for one request at a time and preempt_wait_s set, a short
    request arriving while a long one runs pre-empts it: the short one
    finishes first, the long one still runs all its steps."""
    srv = cg.Server(chunk_steps=5, preempt_wait_s=0.05, **capacity(1, L=16, n_cilia=4, max_replicas=1))
    long_id = srv.submit(request_cfg(16, 4, seed=1), 400, seed=5)
    t0 = time.time()
    while srv.info(long_id)["state"] != cg.REQ_RESIDENT and time.time() - t0 < 60:
        time.sleep(0.002)
    short_id = srv.submit(request_cfg(16, 0, seed=2), 10, seed=6)
    s_info = srv.wait(short_id, 300)
    l_info = srv.wait(long_id, 300)
    assert s_info["state"] == l_info["state"] == cg.REQ_DONE
    assert s_info["steps"] == 10 and l_info["steps"] == 400
    assert l_info["preemptions"] >= 1 and s_info["preemptions"] == 0
    assert s_info["t_done"] < l_info["t_done"]
    srv.close()
