"""Output writers against the reference's own files on the same state.

tests/golden/writers10.npz holds what the reference's writers wrote on the
clami10 run of tests/golden/clami10.npz (same seed, draws and MD step):
mpcd.san (MPCD::debug, src/libcilia/mpcd.cpp:404-467: a row from
Simulation's constructor and one after steps 2 and 4), volvox.san and
volvox.xyz (Clami::writedata, src/clami.cpp:208-284, after steps 2 and 4,
as Simulation::run writes after a measure interval).  The GPU Simulation
replays the run on the recorded draws and writes through
cilia_sim_writedata in a scratch directory; the files are compared value by
value: both sides print six significant digits, so values agree to 1e-5
relative, except the total momentum, which is round-off (below 1e-12) on
both sides; the analysis reader (analysis.load_san) reads both.
"""
import numpy as np
import pytest

import analysis
import cilia_gpu as cg
from conftest import GOLDEN, golden

pytestmark = pytest.mark.gpu


def rows(text):
    return np.array([[float(x) for x in ln.split()] for ln in text.strip().splitlines()])


def xyz_values(text):
    vals = []
    for ln in text.strip().splitlines():
        for tok in ln.split():
            try:
                vals.append(float(tok))
            except ValueError:
                pass
    return np.array(vals)


@pytest.mark.parametrize("arith", [cg.MD_DF, cg.MD_F64])
def test_writers_match_reference_files(tmp_path, monkeypatch, arith):
    g = golden("clami10")
    w = golden("writers10")
    monkeypatch.chdir(tmp_path)
    text = open(f"{GOLDEN}/cases/clami10.cfg").read()
    seed, steps, ststep = w["params"]
    s = cg.Sim(text, precision=cg.MPCD_FP64, ststep=float(ststep), create_fluid=False, md_arith=arith)
    e = s.engine
    e.set_fluid(g["step0_fluid_pos"], g["step0_fluid_vel"])
    e.shift = g["shift_0"]
    s.writedata(objects=False, debug=True)  # Simulation's constructor: MPCD::debug
    writes = set(int(x) for x in w["writes"])
    for k in range(1, int(steps) + 1):
        s.next_tstep(g[f"shift_{k}"], g[f"gamma_{k}"], g[f"axis_{k}"])
        if k in writes:
            s.writedata(objects=True, debug=True)
    assert np.array_equal(e.shift, w[f"shift_{int(steps)}"])
    s.close()
    ref = {k[5:]: w[k].tobytes().decode() for k in w if k.startswith("file_")}
    mine = {name: (tmp_path / name).read_text() for name in ref}
    # mpcd.san: time, dissipated energy since the last clear, N, M, momentum / M, kT
    a, b = rows(mine["mpcd.san"]), rows(ref["mpcd.san"])
    assert a.shape == b.shape == (3, 8)
    for c in (0, 1, 2, 3, 7):
        np.testing.assert_allclose(a[:, c], b[:, c], rtol=1e-5, atol=1e-12)
    assert np.abs(a[:, 4:7]).max() < 1e-12 and np.abs(b[:, 4:7]).max() < 1e-12
    # volvox.san: time, centre of mass, its velocity, body frame n, b, p, dissipated power
    a, b = rows(mine["volvox.san"]), rows(ref["volvox.san"])
    assert a.shape == b.shape == (2, 17)
    np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-9)
    sa = analysis.load_san(tmp_path / "volvox.san")
    assert np.allclose(sa["power"], b[:, 16], rtol=1e-5)
    # volvox.xyz: the cilia's beads of every other row, two frames
    a, b = xyz_values(mine["volvox.xyz"]), xyz_values(ref["volvox.xyz"])
    assert a.shape == b.shape
    np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-9)
