"""The drop-in executable `cilia sim.cfg` (src/main.cpp:117-148) and the
checkpoint files it and `Simulation` write (src/simulation.cpp:354-380:
<object>.dat per MD object, fluid_n.dat, mpcd.dat; the cfg rewritten with the
new globalt, src/main.cpp:95-96).

* The executable runs a small ciliated sphere to `desiredt`, writes the
  checkpoint and the cfg, and a second invocation resumes from those files.
* A resumed Simulation holds exactly the state that was saved (fluid to
  1e-13: positions go through wrapped absolute coordinates; beads, cilia beat
  state and rest lengths, grid shift and time exactly), and for stand-alone
  objects it advances like the original: with the same injected randomness
  both agree to 1e-10 (float64) / 1e-4 (float32) after three more MPC steps.
"""
import os
import subprocess

import numpy as np
import pytest

import cilia_gpu as cg
import simcfg

pytestmark = pytest.mark.gpu

EXE = os.path.join(os.path.dirname(cg.LIB_PATH), "cilia")


def small_swimmer(desiredt):
    cfg = simcfg.swimmer_config(12, radius=3.0, n_cilia=6, rodlength=6, seed=4, ststep=0.002, name="cli")
    cfg["desiredt"] = float(desiredt)
    cfg["seed"] = 17
    return cfg


def test_executable_runs_and_resumes(tmp_path):
    path = tmp_path / "sim.cfg"
    path.write_text(simcfg.dumps(small_swimmer(0.5)))
    r = subprocess.run([EXE, "sim.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    for f in ("fluid_n.dat", "mpcd.dat", "mpcd.san", "inital_randi.dat", "end_randi.dat"):
        assert (tmp_path / f).exists(), f
    objs = [f for f in os.listdir(tmp_path) if f.endswith(".dat") and f not in ("fluid_n.dat", "mpcd.dat")]
    assert len(objs) >= 2, objs  # the sphere and the cilia
    # the run advances in chunks of the measure interval (src/simulation.cpp:112-118)
    cfg = simcfg.load(str(path))
    g1 = float(cfg["globalt"])
    assert g1 >= 0.5 - 1e-9
    n_first = int(open(tmp_path / "fluid_n.dat").readline().split()[1])
    assert n_first == 12 ** 3 * 10
    # resume: raise desiredt, run again from the written files
    cfg["desiredt"] = g1 + 0.1
    path.write_text(simcfg.dumps(cfg))
    r = subprocess.run([EXE, "sim.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert float(simcfg.load(str(path))["globalt"]) >= g1 + 0.1 - 1e-9
    assert "T=" + str(g1)[:3] in r.stdout or "T=" in r.stdout
    san = np.loadtxt(tmp_path / "mpcd.san", ndmin=2)
    assert len(san) >= 2 and np.all(np.abs(san[:, 7] - 1.0) < 0.1)  # kT column of both runs
    # the swimmer's <name>.san (Clami::writedata) read by the analysis restatement
    import analysis

    swim = [f for f in os.listdir(tmp_path) if f.endswith(".san") and f not in ("mpcd.san", "temp.san")]
    assert swim, os.listdir(tmp_path)
    d = analysis.load_san(tmp_path / swim[0])
    assert len(d["time"]) >= 2 and np.all(np.diff(d["time"]) > 0)
    N, B, P = analysis.orientation(d)
    assert np.allclose(np.linalg.norm(N, axis=1), 1.0) and np.allclose(np.linalg.norm(P, axis=1), 1.0)
    assert np.all(np.isfinite(d["vx"])) and np.all(np.isfinite(d["power"]))


def _state(s):
    e = s.engine
    p, v = e.fluid()
    bp, bv = s.beads()
    return dict(p=p, v=v, bp=bp, bv=bv, shift=e.shift.copy(), t=e.time)


def _cilia(s, nc):
    st = np.zeros(2 * nc)
    nl, ol = np.zeros(4096), np.zeros(4096)  # bond tables (sum of rodlengths), sized generously
    s.engine._ck(cg.lib().mpcd_get_cilia(s.engine._h, nc, cg._dp(st), cg._dp(nl), cg._dp(ol)), "get_cilia")
    return st.reshape(nc, 2), nl, ol


def _inject(n, ncell, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        ax = rng.normal(size=(ncell, 3))
        ax /= np.linalg.norm(ax, axis=1, keepdims=True)
        out.append((rng.uniform(0, 1, 3), rng.gamma(13.5, size=ncell), ax))
    return out


def _save_and_resume(tmp_path, text, precision, nc, L, steps=4):
    a = cg.Sim(text, precision=precision, seed=9, ststep=0.002)
    for _ in range(steps):
        a.next_tstep()
    a.save()
    a.write_cfg(str(tmp_path / "sim.cfg"))
    saved = _state(a)
    b = cg.Sim(str(tmp_path / "sim.cfg"), is_text=False, precision=precision, seed=9, ststep=0.002, read_files=True)
    got = _state(b)
    d = got["p"] - saved["p"]
    d -= np.round(d / L) * L
    assert np.abs(d).max() < 1e-13
    assert np.array_equal(got["v"], saved["v"])
    assert np.array_equal(got["bp"], saved["bp"]) and np.array_equal(got["bv"], saved["bv"])
    assert np.array_equal(got["shift"], saved["shift"]) and got["t"] == saved["t"]
    (sa, _, ola), (sb, _, olb) = _cilia(a, nc), _cilia(b, nc)
    assert np.array_equal(sa, sb) and np.array_equal(ola, olb)
    return a, b


@pytest.mark.parametrize("precision", [cg.MPCD_FP64, cg.MPCD_FP32])
def test_checkpoint_restores_the_swimmer(tmp_path, monkeypatch, precision):
    """A Clami: the resumed state equals the saved one.  (Its attachment
    springs are rebuilt from the loaded positions on construction, as
    Clami::init_attachment_springs does in the reference (src/clami.cpp:
    152-183), so a resumed swimmer is not expected to continue bitwise.)"""
    monkeypatch.chdir(tmp_path)
    a, b = _save_and_resume(tmp_path, simcfg.dumps(small_swimmer(10.0)), precision, nc=6, L=12.0)
    a.close()
    b.close()


@pytest.mark.parametrize("precision", [cg.MPCD_FP64, cg.MPCD_FP32])
def test_resumed_run_continues_like_the_original(tmp_path, monkeypatch, precision):
    """Stand-alone Sphere, Cilia and ConstantBeatCilia (the objects8 case):
    saved, resumed, then both advanced with the same injected randomness."""
    from conftest import GOLDEN

    monkeypatch.chdir(tmp_path)
    text = open(f"{GOLDEN}/cases/objects8.cfg").read()
    a, b = _save_and_resume(tmp_path, text, precision, nc=2, L=8.0)
    for sh, g, ax in _inject(3, a.engine.ncell, seed=5):
        a.next_tstep(sh, g, ax)
        b.next_tstep(sh, g, ax)
    fa, fb = _state(a), _state(b)
    tol = 1e-10 if precision == cg.MPCD_FP64 else 1e-4
    d = fa["p"] - fb["p"]
    d -= np.round(d / 8.0) * 8.0
    assert np.abs(d).max() < tol and np.abs(fa["v"] - fb["v"]).max() < 10 * tol
    assert np.abs(fa["bp"] - fb["bp"]).max() < tol
    a.close()
    b.close()
