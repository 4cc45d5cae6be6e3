"""Benchmark: MPCD particle-steps/s of the microswimmer hot path on GB300.

Default workload (N = 1): `swimmer64` - 64^3 periodic cells x 10 fluid
particles (2,621,440) plus a ciliated sphere (Clami, radius 8, 100 cilia of
3 x 15 beads on a Fibonacci lattice; 5,143 beads), 50 MD velocity-Verlet
substeps per MPC step, the plain float64 method.  One step = one full MPC
step: collision, all MD substeps, grid shift, streaming and binning.

value  : (fluid + beads) x steps / device time of the timed steps (CUDA events
         on the engine's stream; the L2 is flushed between steps).  The MD
         substeps run in double-float arithmetic (the float64 path's default,
         `md_arith`); `ieee_fp64` is the same workload with IEEE float64 MD
         (the pair kernel: each spring pair evaluated once).
e2e    : the same metric through the C ABI with host buffers over a fixed
         window of 200 steps: the fluid and swimmer uploaded from host memory,
         every step followed by an observables read-back, the final state
         downloaded (wall clock).  The one-time upload / download and the
         steady per-step rate are reported beside it.
roofline: the fluid collide+stream kernel against the measured HBM copy
         bandwidth; algorithmic bytes per particle-step = read + write of the
         reference's particle state (float64: 3 position + 4 velocity/mass
         doubles = 56 B each way, 112 B; float32 split: 2 float4 = 64 B); the
         96 B this build's float64 state moves (no mass column) beside it.
cpu_baseline: the C restatement of the reference (oracle/) with OpenMP on the
         host cores, on a bounded sample of the same workload.
plain_fluid: the 32^3 periodic fluid (327,680 particles, no swimmer).
batched: the 64-replica mixed-size ensemble (box edges 16..48, 0-64 cilia)
         advanced together by the replica batch (float32 split, CUDA graphs,
         autotuned launch configuration), 1000 MPC steps timed, beside the
         same replicas run one at a time through the single-box engine.
serving: 500 swimmer-run requests (box edges 16..64, 0-200 cilia, steps
         log-uniform in 500..20000) arriving as a Poisson process, served by
         continuous batching: p50 / p99 completion latency and throughput.
large_swimmer: the 128^3 box with a radius-16 Clami of 400 cilia (3 x 20
         beads) in float32 split precision, beside the float64 plain path, and
         its observables against the float64 oracle run on the same initial
         state and the same random draws.

--impl reference runs that CPU restatement alone (the reference's own
sources are not available where this runs) and prints its line.
--ensemble-only --no-plain runs only the replica batch (the command of the
batch fluid pass's ncu profile).
Multi-GPU: replicas only - every rank advances its own independent box.
"""
from __future__ import annotations

import argparse
import gc
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "multi-ciliated-microswimmers_gb300")
for _p in (PKG, os.path.join(REPO, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import simcfg  # noqa: E402

METRIC = "MPCD particle-steps/s"
# DRAM bytes (read + write) per fluid particle of one fluid_step launch, from
# one ncu capture on swimmer64 (profiles/fluid_step_swimmer64.md); the traffic
# grows in proportion to the particles, so it is scaled to the workload.
TRAFFIC_B_PER_PARTICLE = {"fp64": 98.9, "fp32": 48.7}
# the replica batch's fluid pass on the 64-replica ensemble
# (profiles/batch_fluid_ensemble64.md: 2,389.7 MB for 34,273,280 particles)
BATCH_TRAFFIC_B_PER_PARTICLE = 2389.7e6 / 34273280
# FP64 pipe of the same captures (sm__pipe_fp64_cycles_active, of peak, active):
# the float64 fluid step is bound by it, not by HBM
FP64_PIPE_ACTIVE = {"fp64": 0.824, "fp32": 0.014}
# algorithmic bytes per particle-step: read + write of the reference's state
# (float64: 3 position + 4 velocity/mass doubles; float32 split: two float4)
BYTES_PER_PARTICLE = {"fp64": 112, "fp32": 64}
# what this build's float64 layout moves (no mass column: 3 offsets + 3 velocities)
STATE_BYTES_PER_PARTICLE = {"fp64": 96, "fp32": 64}
UNIT = "particle-steps/s"
E2E_STEPS = 200


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock and throttle sampling during the timed region."""

    def __init__(self, device=0):
        self.device = device
        self.samples = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.3)  # the first sample lands before the timed region starts
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[4 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def workload_cfg(name, seed):
    cfg = simcfg.baseline_config(name, seed=seed)
    cfg["seed"] = int(seed)
    return cfg


MD_ARITH_NAMES = {
    0: "float64",
    1: "split (float springs on hi/lo position pairs)",
    2: "double-float (pairs of floats, 48-bit significand; integer cell + offset coordinates)",
    3: "float springs on double-float positions (split arithmetic; integer cell + offset coordinates)",
    4: "float64, each spring pair evaluated once (pair kernel)",
    5: "double-float, each spring pair evaluated once (pair kernel; integer cell + offset coordinates)",
}


def describe(name, nf, nb, precision):
    if name == "swimmer64":
        geo = "64^3 cells x 10 fluid, Clami R=8 with 100 cilia (3x15 beads) on a Fibonacci lattice, 50 MD substeps"
    elif name == "swimmer128":
        geo = "128^3 cells x 10 fluid, Clami R=16 with 400 cilia (3x20 beads), 50 MD substeps"
    else:
        geo = "32^3 cells x 10 fluid, periodic, no swimmer"
    return f"{name}: {geo}; {nf} fluid + {nb} beads; {precision}"


def arm_config(args, nf, nb):
    """The `config` both arms print for the same workload."""
    prec = "float64 plain" if args.precision == "fp64" else "float32 split"
    return {"workload": describe(args.workload, nf, nb, prec),
            "l2": "flushed between timed steps (256 MB write, outside the timed events)",
            "parallelism": f"replicas{args.gpus}"}


# ------------------------------------------------------------------ GPU arm --

def run_gpu(args, rank=0, md_arith=None, steps=None, workload=None, precision=None):
    import cilia_gpu as cg

    precision = precision or args.precision
    workload = workload or args.workload
    prec = cg.MPCD_FP64 if precision == "fp64" else cg.MPCD_FP32
    cfg = workload_cfg(workload, seed=1000 + rank)
    text = simcfg.dumps(cfg)
    if md_arith is None:  # --md-arith for the main line (profiling runs of one MD kernel)
        md_arith = {"auto": cg.MD_AUTO, "pair": cg.MD_PAIR, "pair-df": cg.MD_PAIR_DF}[getattr(args, "md_arith", "auto")]
    sim = cg.Sim(text, precision=prec, seed=1000 + rank, device=args.device, md_arith=md_arith)
    steps = args.steps if steps is None else steps
    eng = sim.engine
    nf = len(eng.fluid()[1]) if args.verify_counts else int(cfg["sizex"]) ** 3 * 10
    nb = sim.nbeads
    ntot = nf + nb
    eng.run(args.warmup)
    eng.sync()
    launches0 = eng.launch_count()
    with ClockSampler(args.device) as clk:
        step_ms = eng.timed_run(steps, flush_l2=True)
    launches = eng.launch_count() - launches0
    total_s = float(step_ms.sum()) / 1e3
    value = ntot * steps / total_s
    # per-kernel times on a short profiled run (events around every launch)
    prof_steps = min(steps, 20)
    eng.set_profiling(True)
    eng.timed_run(prof_steps, flush_l2=True)
    kt = {k: eng.kernel_time(i) for k, i in (("cell", cg.K_CELL), ("fluid", cg.K_FLUID), ("bead", cg.K_BEAD),
                                              ("md", cg.K_MD), ("sort", cg.K_SORT))}
    eng.set_profiling(False)
    obs = eng.observables()
    md_arith = eng.md_layout()["arith"] if nb else None
    sim.close()
    return dict(value=value, ms_per_step=1e3 * total_s / steps, nf=nf, nb=nb, kernels=kt,
                launches=launches, clocks=clk.summary(), kT=obs["kT"], step_ms=step_ms, prof_steps=prof_steps,
                md_arith=md_arith)


def roofline(nf, kernels, precision):
    """The fluid collide + stream + bin kernel against the measured HBM copy bandwidth."""
    hbm, peak_kind = peaks()
    fl_ms, fl_n = kernels["fluid"]
    avg_ms = fl_ms / max(fl_n, 1)
    bpp = BYTES_PER_PARTICLE[precision]
    achieved = nf * bpp / (avg_ms * 1e-3) / 1e9
    state = nf * STATE_BYTES_PER_PARTICLE[precision] / (avg_ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": TRAFFIC_B_PER_PARTICLE[precision] * nf,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, swimmer64 capture, scaled by "
                              "particles", "peak_kind": peak_kind, "kernel": "fluid_step (collide + stream + bin)",
            "bytes_per_particle_step": bpp, "avg_launch_ms": avg_ms,
            "state_bytes_per_particle_step": STATE_BYTES_PER_PARTICLE[precision], "frac_state_bytes": state / hbm,
            "fp64_pipe_active": FP64_PIPE_ACTIVE[precision],
            "fp64_pipe_source": "ncu sm__pipe_fp64_cycles_active, swimmer64 capture (the float64 kernel's bound)"}


def run_e2e(args):
    """Through the C ABI with host buffers (the fluid arrays page-locked with
    mpcd_pin_host), over a fixed window of E2E_STEPS
    steps: upload of the fluid (the swimmer is built on the host and uploaded
    with the Sim), every step followed by an observables read-back (enqueued
    with mpcd_observables_async, collected inside the window), final download
    of fluid and beads; wall clock."""
    import cilia_gpu as cg

    assert E2E_STEPS <= cg.OBS_RING
    prec = cg.MPCD_FP64 if args.precision == "fp64" else cg.MPCD_FP32
    cfg = workload_cfg(args.workload, seed=77)
    L = int(cfg["sizex"])
    rng = np.random.default_rng(5)
    nf = L ** 3 * 10
    pos = rng.uniform(0, L, (nf, 3))
    vel = rng.normal(size=(nf, 3))
    vel -= vel.mean(axis=0)
    sim = cg.Sim(simcfg.dumps(cfg), precision=prec, seed=77, create_fluid=False, device=args.device)
    eng = sim.engine
    nb = sim.nbeads
    bpos, bvel = sim.beads()
    # the host side of the fluid copies lives in page-locked buffers (pinned
    # once, outside the window), so both directions run as direct DMA
    pout, vout = np.empty_like(pos), np.empty_like(vel)
    pinned = [eng.pin(a) for a in (pos, vel, pout, vout)]
    # one untimed pass of the same calls (first-use costs of the host pages
    # and the CUDA driver's copy path stay out of the window)
    eng.set_fluid(pos, vel)
    for _ in range(3):
        eng.step()
        eng.observables_result(eng.observables_async())
    eng.fluid(out=(pout, vout))
    # no garbage-collector pass inside the window (after the other bench legs
    # one took milliseconds of host time)
    gc.collect()
    gc.disable()
    try:
        t0 = time.perf_counter()
        eng.set_fluid(pos, vel)
        t1 = time.perf_counter()
        # each step's observables are enqueued behind it and all are collected
        # inside the window: the read-backs are all done, the host just does
        # not stall the next step on them
        tickets = []
        for _ in range(E2E_STEPS):
            eng.step()
            tickets.append(eng.observables_async())
        obs = [eng.observables_result(t) for t in tickets]
        t2 = time.perf_counter()
        p, v = eng.fluid(out=(pout, vout))
        bp, bv = sim.beads()
        t3 = time.perf_counter()
    finally:
        gc.enable()
    if not all(np.isfinite(o["kT"]) for o in obs):
        raise RuntimeError("non-finite observables in the end-to-end window")
    for a in pinned:
        eng.unpin(a)
    sim.close()
    up = pos.nbytes + vel.nbytes + bpos.nbytes + bvel.nbytes
    down = p.nbytes + v.nbytes + bp.nbytes + bv.nbytes
    obs_bytes = 80
    ntot = nf + nb
    return dict(value=ntot * E2E_STEPS / (t3 - t0), h2d=up / E2E_STEPS, d2h=down / E2E_STEPS + obs_bytes,
                steady=ntot * E2E_STEPS / (t2 - t1), upload_s=t1 - t0, download_s=t3 - t2, up=up, down=down,
                step_ms=1e3 * (t2 - t1) / E2E_STEPS)


def run_plain(args):
    """The 32^3 periodic fluid (the plain-fluid workload), float64 and float32 split."""
    out = {}
    for prec in ("fp64", "fp32"):
        g = run_gpu(args, workload="plain32", precision=prec, steps=max(20, min(args.steps, 200)))
        rf = roofline(g["nf"], g["kernels"], prec)
        out[prec] = {"value": g["value"], "ms_per_step": g["ms_per_step"], "kT": g["kT"],
                     "fluid_kernel_ms": rf["avg_launch_ms"], "roofline_frac": rf["frac"],
                     "bytes_per_particle_step": rf["bytes_per_particle_step"]}
    out["workload"] = "plain32: 32^3 cells x 10 fluid (327680 particles), h = 0.1, no swimmer, L2 flushed"
    return out


# --------------------------------------------------------- batched ensemble --

def run_ensemble(args, n=64, steps=1000, plain=True, stage_steps=20):
    """64 uneven replicas (box edge in {16..48}, sphere radius edge/8, 0-64
    cilia of rodlength 10-15) advanced together by the replica batch, FP32
    split, `steps` MPC steps timed; beside it (plain=True) the same replicas
    run one at a time through the single-box engine (the plain path), FP64
    and FP32.  With plain=False and steps=0 only the stage timer runs
    (`stage_steps` serialised steps): the command the batch fluid pass is
    profiled with."""
    import cilia_gpu as cg

    specs = simcfg.ensemble_specs(n, seed=11)
    b = cg.Batch.for_specs(specs, device=args.device)
    ids, parts = [], 0
    single = {"fp64": [0.0, 0.0], "fp32": [0.0, 0.0]}  # particle-steps, ms
    for sp in specs:
        text = simcfg.dumps(simcfg.swimmer_config(sp["L"], radius=sp["radius"], n_cilia=sp["n_cilia"],
                                                  rodlength=sp["rodlength"], seed=sp["seed"]))
        for prec, key in ((cg.MPCD_FP64, "fp64"), (cg.MPCD_FP32, "fp32")):
            if key == "fp64" and not plain:
                continue
            s = cg.Sim(text, precision=prec, ststep=0.002, seed=sp["seed"], device=args.device)
            npart = 10 * sp["L"] ** 3 + s.nbeads
            if plain:
                s.engine.run(3)
                ms = s.engine.timed_run(5, flush_l2=True)
                single[key][0] += npart * 5
                single[key][1] += float(ms.sum())
            if key == "fp32":
                r = b.add_engine(s.engine)
                b.admit(r)
                ids.append(r)
                parts += npart
            s.close()
    for r in ids:
        b.set_steps(r, 10 ** 9)
    if steps == 0:
        b.set_md_layout(1, 512)
        b.set_tuning(fluid_threads=256, fluid_blocks=0, cell_threads=256, cell_blocks=0, sort_interval=100)
        stage = b.stage_times(stage_steps)
        b.close()
        return {"stage_ms_per_step": stage, "particles": parts, "replicas": len(ids)}
    tuning = b.autotune(trial_steps=50)
    stage = b.stage_times(stage_steps)
    for r in ids:
        b.set_steps(r, steps)
    l0 = b.launch_count()
    with ClockSampler(args.device) as clk:
        ms = b.timed_run(steps)
    launches = b.launch_count() - l0
    value = parts * steps / (ms / 1e3)
    kts, mom, errs = [], [], 0
    for r in ids:
        st = b.status(r)
        errs += int(st["err"] != 0 or st["steps"] < steps)
        o = b.observables(r)
        kts.append(o["kT"])
        mom.append(float(np.abs(o["momentum"]).max()))
    nf_tot = sum(10 * sp["L"] ** 3 for sp in specs)
    hbm, peak_kind = peaks()
    achieved = nf_tot * 64 / (stage["fluid"] * 1e-3) / 1e9
    plain64 = single["fp64"][0] / (single["fp64"][1] / 1e3)
    plain32 = single["fp32"][0] / (single["fp32"][1] / 1e3)
    step_bytes = value / parts * nf_tot * 64 / 1e9  # fluid state bytes per second of the whole timed step
    b.close()
    return {
        "workload": f"ensemble{n}: {n} replicas, box edge uniform in {{16,24,32,40,48}} x 10 fluid/cell, "
                    f"Clami radius edge/8 with 0-64 cilia of 3x(10-15) beads, 50 MD substeps, float32 split; "
                    f"{parts} particles (fluid + beads)",
        "metric": METRIC, "value": value, "unit": UNIT, "steps": steps, "ms_per_step": ms / steps,
        "l2": "inputs (0.9 GB of fluid state) larger than L2", "gpu_launches": launches,
        "plain_single_run": {"fp64": plain64, "fp32": plain32,
                             "how": "each replica alone through the single-box engine, 5 timed steps, L2 flushed"},
        "speedup_vs_plain_fp64": value / plain64, "speedup_vs_single_fp32": value / plain32,
        "step_hbm_frac": step_bytes / hbm,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": BATCH_TRAFFIC_B_PER_PARTICLE * nf_tot,
                     "traffic_frac": BATCH_TRAFFIC_B_PER_PARTICLE * nf_tot / (stage["fluid"] * 1e-3) / 1e9 / hbm,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the same ensemble "
                                       "(profiles/batch_fluid_ensemble64.md), scaled by particles",
                     "peak_kind": peak_kind, "kernel": "batch fluid_step (collide + stream + bin), stages serialised",
                     "bytes_per_particle_step": 64, "avg_launch_ms": stage["fluid"]},
        "stage_ms_per_step": stage, "tuning": tuning, "clocks": clk.summary(),
        "kT": {"min": min(kts), "max": max(kts), "mean": float(np.mean(kts))},
        "max_momentum_per_mass": max(mom), "replicas_with_errors": errs,
    }


# ----------------------------------------------------------------- serving --

def run_serving(args, n=500, steps_range=(500, 20000), load=0.8, seed=21):
    """Continuous batching of swimmer runs: Poisson arrivals of requests with
    box edge uniform in 16..64 (10 fluid per cell), 0-200 cilia of rodlength
    15 on a sphere of radius min(8, edge/4) (a radius-edge/8 sphere carrying
    more than about 70 cilia goes numerically unstable within a few hundred
    steps in the reference's own arithmetic), step counts log-uniform in
    steps_range, float32 split; the arrival rate offers `load` x an estimated
    throughput.  Reports completion latency (submit -> done) percentiles and
    throughput."""
    import cilia_gpu as cg

    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(n):
        L = int(rng.integers(16, 65))
        nc = int(rng.integers(0, 201))
        st = int(round(math.exp(rng.uniform(math.log(steps_range[0]), math.log(steps_range[1])))))
        reqs.append((L, nc, st, 1000 + k))
    e_l3 = float(np.mean([x ** 3 for x in range(16, 65)]))
    mean_particles = 10 * e_l3 + 643 + 45 * 100
    mean_steps = (steps_range[1] - steps_range[0]) / math.log(steps_range[1] / steps_range[0])
    est_throughput = 1.5e10  # particle-steps/s of a full batch (ensemble measurement)
    rate = load * est_throughput / (mean_particles * mean_steps)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
    # capacity for about 64 average requests resident, budget 60 % of it (admission by footprint)
    cap_req = 64
    caps = dict(max_replicas=cap_req + 16, max_particles=int(cap_req * 10 * e_l3 * 1.1) + 64 * 8192,
                max_cells=int(cap_req * e_l3 * 1.1) + 64 * 2048, max_slots=cap_req * 2 * 5200 + 40 * 2048,
                max_springs=cap_req * 14 * 5200, max_halo=cap_req * 6 * 5200 + 4096, max_cilia=cap_req * 200,
                max_bonds=cap_req * 200 * 15, md_lanes=1, md_tile=1024)
    # the device bytes of the whole capacity; requests are admitted while the
    # sum of their footprints stays within 60 % of it
    cap_bytes = cg.lib().mpcd_batch_estimate(None, caps["max_particles"], caps["max_cells"], cap_req * 5200,
                                             caps["max_springs"], caps["max_cilia"], caps["max_bonds"])
    budget = int(0.6 * cap_bytes)
    srv = cg.Server(budget_bytes=budget, chunk_steps=25, prep_threads=4, device=args.device, **caps)
    texts = {}
    t0 = time.perf_counter()
    ids = []
    for (L, nc, st, sd), ta in zip(reqs, arrivals):
        key = (L, nc)
        if key not in texts:
            texts[key] = simcfg.dumps(simcfg.swimmer_config(L, radius=min(8.0, L / 4.0), n_cilia=nc, rodlength=15,
                                                            seed=sd))
        dt = t0 + ta - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        ids.append(srv.submit(texts[key], st, seed=sd))
    srv.drain(3600)
    wall = time.perf_counter() - t0
    st = srv.stats()
    infos = [srv.info(i) for i in ids]
    errors = sorted({f"{srv.error(i)} (bits {inf['err']}, L {r[0]}, cilia {r[1]})"
                     for i, inf, r in zip(ids, infos, reqs) if inf["state"] != cg.REQ_DONE})
    srv.close()
    done = [i for i in infos if i["state"] == cg.REQ_DONE]
    return {
        "workload": f"serving: {n} swimmer runs, Poisson arrivals at {rate:.2f}/s, box edge uniform 16..64 x 10 "
                    f"fluid/cell, sphere radius min(8, edge/4) with 0-200 cilia of 3x15 beads, steps log-uniform "
                    f"{steps_range[0]}..{steps_range[1]}, float32 split",
        "metric": METRIC, "value": st["throughput"], "unit": UNIT, "p50_s": st["p50_s"], "p99_s": st["p99_s"],
        "mean_s": st["mean_s"], "max_s": st["max_s"], "completed": st["completed"], "failed": st["failed"],
        "wall_s": wall, "busy_s": st["busy_s"], "particle_steps": st["particle_steps"],
        "peak_resident": st["peak_resident"], "peak_resident_gb": st["peak_resident_bytes"] / 1e9,
        "budget_gb": budget / 1e9, "gpu_launches": st["gpu_launches"],
        "queue_wait_p50_s": float(np.median([i["t_admit"] - i["t_submit"] for i in done])) if done else None,
        "kT_range": [min(i["obs"]["kT"] for i in done), max(i["obs"]["kT"] for i in done)] if done else None,
        "errors": errors[:12],
    }


# ------------------------------------------------------- large swimmer (c2) --

def body_axis(bp):
    """The swimmer's body axis n = sphere bead 1 - bead 0 (Clami::writedata), normalised."""
    n = bp[1] - bp[0]
    return n / np.linalg.norm(n)


def vacf(v0, v):
    """Normalised fluid velocity autocorrelation <v(0).v(t)> / <v(0).v(0)>."""
    return float(np.einsum("ij,ij->", v0, v) / np.einsum("ij,ij->", v0, v0))


def run_large(args, steps=200, seed=2024, oracle_steps=20):
    """swimmer128 (128^3 cells x 10 fluid, Clami R=16 with 400 cilia of 3x20
    beads) in float32 split precision, timed, beside the float64 plain path.
    Then the precision statement: the float32 path run on the float64
    oracle's recorded draws (grid shift, Gamma variates, rotation axes) from
    the oracle's own initial state for `oracle_steps` steps, its observables
    against the oracle's: fluid temperature, the fluid velocity
    autocorrelation, the swimmer's centre-of-mass velocity and speed, and the
    rotation rate of its body axis."""
    import cilia_gpu as cg
    from oracle import build_from_cfg

    cfg = workload_cfg("swimmer128", seed=seed)
    text = simcfg.dumps(cfg)
    res = {}
    for prec, key in ((cg.MPCD_FP32, "fp32"), (cg.MPCD_FP64, "fp64")):
        sim = cg.Sim(text, precision=prec, seed=seed, device=args.device)
        eng = sim.engine
        nf = int(cfg["sizex"]) ** 3 * 10
        nb = sim.nbeads
        eng.run(3)
        ms = eng.timed_run(steps, flush_l2=True)
        lay = eng.md_layout()
        res[key] = dict(value=(nf + nb) * steps / (float(ms.sum()) / 1e3), ms_per_step=float(ms.mean()), nf=nf,
                        nb=nb, md_lanes=lay["lanes"], md_tile=lay["tile"], md_arith=MD_ARITH_NAMES[lay["arith"]])
        sim.close()
    # float32 split on the oracle's draws against the float64 oracle
    t0 = time.perf_counter()
    o = build_from_cfg(cfg, seed=seed, ststep=0.002)
    o.set_threads(os.cpu_count() or 1)
    sim = cg.Sim(text, precision=cg.MPCD_FP32, seed=seed, create_fluid=False, device=args.device)
    eng = sim.engine
    p0, v0 = o.fluid()
    eng.set_fluid(p0, v0)
    eng.shift = o.shift
    ob0, _ = o.beads()
    gb0, _ = sim.beads()
    dt = oracle_steps * float(cfg["tstep"])
    for _ in range(oracle_steps):
        rs, rg, ra, _ = o.step(record=True)
        # a particle within float rounding of a cell face can fill a cell the
        # float64 oracle left with one particle: no Gamma variate was drawn
        # there; such a cell takes the mean of a two-particle cell's Gamma law
        rg = np.where(rg < 0.0, 1.5, rg)
        sim.next_tstep(rs, rg, ra)
    _, vg = eng.fluid()
    _, vo = o.fluid()
    gb, gv = sim.beads()
    ob, ov = o.beads()
    sim.close()
    ang = {}
    for k, (b0, b1) in (("fp32", (gb0, gb)), ("oracle", (ob0, ob))):
        c = float(np.clip(np.dot(body_axis(b0), body_axis(b1)), -1.0, 1.0))
        ang[k] = math.acos(c) / dt
    vc_g, vc_o = gv.mean(axis=0), ov.mean(axis=0)
    stats = {
        "steps": oracle_steps, "oracle_s": time.perf_counter() - t0,
        "fluid_T": [float((vg ** 2).sum() / (3 * len(vg))), float((vo ** 2).sum() / (3 * len(vo)))],
        "vacf": [vacf(v0, vg), vacf(v0, vo)],
        "swimmer_v_cm": [vc_g.tolist(), vc_o.tolist()],
        "swimmer_v_cm_err": float(np.linalg.norm(vc_g - vc_o)),
        "swimmer_speed": [float(np.linalg.norm(vc_g)), float(np.linalg.norm(vc_o))],
        "rotation_rate": [ang["fp32"], ang["oracle"]],
        "rotation_rate_err": abs(ang["fp32"] - ang["oracle"]),
        "bead_pos_err_max": float(np.abs(gb - ob).max()),
        "how": "float32 split GPU run on the float64 oracle's recorded grid shifts, Gamma variates and rotation "
               "axes from the oracle's initial state; pairs are [float32 GPU, float64 oracle]",
    }
    stats["fluid_T_err"] = abs(stats["fluid_T"][0] - stats["fluid_T"][1])
    stats["vacf_err"] = abs(stats["vacf"][0] - stats["vacf"][1])
    a, b = res["fp32"], res["fp64"]
    return {
        "workload": describe("swimmer128", a["nf"], a["nb"], "float32 split") + f"; {steps} timed MPC steps",
        "metric": METRIC, "unit": UNIT, "value": a["value"], "ms_per_step": a["ms_per_step"],
        "plain_fp64": {"value": b["value"], "ms_per_step": b["ms_per_step"]},
        "md_layout": {"lanes": a["md_lanes"], "tile": a["md_tile"], "arith": a["md_arith"]},
        "fp32_vs_fp64_oracle": stats,
    }


# ------------------------------------------------------------------ CPU arm --

def run_cpu(args, budget_s=None, threads=None, warmup=1, steps=None):
    """The C restatement on the host cores: `warmup` untimed steps, then
    `steps` timed steps (stopping early once the time budget is spent)."""
    from oracle import build_from_cfg

    cfg = workload_cfg(args.workload, seed=3)
    threads = threads or os.cpu_count() or 1
    s = build_from_cfg(cfg, seed=3)
    s.set_threads(threads)
    nf = s.fluid()[0].shape[0]
    nb = s.bead_count()
    budget = budget_s if budget_s is not None else args.cpu_budget
    steps = steps if steps is not None else args.steps
    for _ in range(max(warmup, 0)):
        s.step()
    n = 0
    t0 = time.perf_counter()
    while n < steps:
        s.step()
        n += 1
        el = time.perf_counter() - t0
        if el >= budget and n >= 2:
            break
    el = time.perf_counter() - t0
    return dict(value=(nf + nb) * n / el, steps=n, seconds=el, threads=threads, nf=nf, nb=nb)


def max_over_ranks(t_rank, dist, device):
    """The slowest rank's ms per step (replicas: every rank runs its own box)."""
    import torch

    t = torch.tensor([t_rank], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_rank, world, t_max_ms):
    """Whole-job particle-steps/s: the units every rank advanced per step, over
    the slowest rank's step time."""
    return units_per_rank * world / (t_max_ms / 1e3)


def clock_ok(c):
    bad = {"hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"}
    return not (set(c.get("reasons", [])) & bad)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="swimmer64", choices=["swimmer64", "swimmer128", "plain32"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--md-arith", default="auto", choices=["auto", "pair", "pair-df"],
                    help="MD arithmetic of the main line (auto: the default; pair: float64 pair kernel)")
    ap.add_argument("--device", type=int, default=None)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true")
    ap.add_argument("--verify-counts", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--ensemble-only", action="store_true")
    ap.add_argument("--no-plain", action="store_true",
                    help="with --ensemble-only: skip the one-at-a-time runs and the timed run (stage timer only)")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-large", action="store_true", help="skip the 128^3 swimmer line")
    ap.add_argument("--serving-only", action="store_true")
    ap.add_argument("--serving-quick", action="store_true", help="60 requests, steps 100..2000")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.device is None:
        args.device = local
    serving_kw = dict(n=60, steps_range=(100, 2000)) if args.serving_quick else {}

    if args.impl == "reference":
        if rank != 0:
            return
        # 300 s at most for the timed steps (the full --steps when they fit)
        r = run_cpu(args, budget_s=max(args.cpu_budget, 300.0), warmup=args.warmup, steps=args.steps)
        line = {"impl": "reference", "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": args.gpus,
                "steps": r["steps"], "warmup": args.warmup, "ms_per_step": 1e3 * r["seconds"] / r["steps"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if args.precision == "fp64" else "f32", "data": "synthetic",
                "config": arm_config(args, r["nf"], r["nb"]),
                "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": r["threads"], "kind": "port",
                                 "sample": f"{r['steps']} MPC steps of the full workload after {args.warmup} "
                                           f"warm-up steps, {r['seconds']:.1f} s, C restatement of the reference "
                                           f"(float64 throughout), OpenMP on {r['threads']} host threads"},
                "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if args.ensemble_only:
        if rank == 0:
            if args.no_plain:
                print(json.dumps(run_ensemble(args, plain=False, steps=0, stage_steps=args.steps)))
            else:
                print(json.dumps(run_ensemble(args)))
        return
    if args.serving_only:
        if rank == 0:
            print(json.dumps(run_serving(args, **serving_kw)))
        return
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(args.device)
        dist.init_process_group("nccl")
        dist.barrier()
    g = run_gpu(args, rank)
    if not clock_ok(g["clocks"]):  # throttled: measure once more
        g = run_gpu(args, rank)
    value_rank = g["value"]
    t_rank = g["ms_per_step"]
    if dist is not None:
        t_max = max_over_ranks(t_rank, dist, f"cuda:{args.device}")
        value = job_value(g["nf"] + g["nb"], world, t_max)
        dist.barrier()
    else:
        t_max = t_rank
        value = value_rank
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32",
        "data": "synthetic",
        "config": arm_config(args, g["nf"], g["nb"]),
        "kernels_ms_per_step": {k: v[0] / max(g["prof_steps"], 1) for k, v in g["kernels"].items()},
        "kT": g["kT"],
    }
    if g["md_arith"] is not None:
        line["md_arith"] = MD_ARITH_NAMES[g["md_arith"]]
    # the end-to-end window before the other legs: after the batch, serving
    # and 128^3 legs in the same process its 126 MB download took 6-12 ms
    # instead of 1.3 ms; and before the CPU baseline, whose OpenMP threads keep
    # spinning for a while after it and slow the host side of the copies
    e = run_e2e(args) if not args.no_extra else None
    # the long nested records first, the short headline figures last (the end
    # of the line is what a truncated log keeps)
    if not args.no_ensemble and args.gpus == 1:
        line["batched"] = run_ensemble(args)
    if not args.no_serving and args.gpus == 1:
        line["serving"] = run_serving(args, **serving_kw)
    if not args.no_large and args.gpus == 1 and args.workload == "swimmer64":
        line["large_swimmer"] = run_large(args)
    if not args.no_extra and args.gpus == 1:
        line["plain_fluid"] = run_plain(args)
    if args.precision == "fp64" and g["nb"] and not args.no_extra:
        # the same workload with the MD substeps in IEEE float64 arithmetic
        import cilia_gpu as cg

        k = max(3, min(args.steps, 100))
        f = run_gpu(args, rank, md_arith=cg.MD_PAIR, steps=k)
        line["ieee_fp64"] = {"value": f["value"], "ms_per_step": f["ms_per_step"],
                             "md_ms_per_step": f["kernels"]["md"][0] / max(f["prof_steps"], 1), "steps": k,
                             "md_arith": MD_ARITH_NAMES[4]}
    line["roofline"] = roofline(g["nf"], g["kernels"], args.precision)
    if e is not None:
        line["e2e"] = {"value": e["value"], "unit": UNIT, "h2d_bytes_per_step": e["h2d"],
                       "d2h_bytes_per_step": e["d2h"], "steps": E2E_STEPS,
                       "steady_value": e["steady"], "steady_ms_per_step": e["step_ms"],
                       "upload_s": e["upload_s"], "download_s": e["download_s"],
                       "upload_bytes": e["up"], "download_bytes": e["down"],
                       "host_buffers": "fluid arrays page-locked (mpcd_pin_host) before the window"}
    if not args.no_cpu:
        c = run_cpu(args)
        line["cpu_baseline"] = {"value": c["value"], "unit": UNIT, "cores": c["threads"], "kind": "port",
                                "sample": f"{c['steps']} MPC steps of {args.workload} ({c['nf']} fluid + "
                                          f"{c['nb']} beads) in {c['seconds']:.1f} s, C restatement, OpenMP"}
    line["gpu_launches"] = g["launches"]
    line["clocks"] = g["clocks"]
    print(json.dumps(line))


if __name__ == "__main__":
    main()
