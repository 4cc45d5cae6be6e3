"""Drop-in resume from checkpoints the reference itself wrote.

tests/golden/resume10.npz holds the files a reference run of the clami10
case leaves behind (Simulation's destructor: fluid_n.dat from Fluid::save,
<object>.dat from MDObject::save / Cilia::save / Sphere::save / Clami::save,
mpcd.dat from MPCD's destructor) and a second reference run started in the
same directory: its loaded state (step0), its recorded draws and its state
after two more steps.  `cilia sim.cfg`'s Simulation (cilia_sim_create with
read_files) is started in a directory holding those files and must

  * load the same state: fluid velocities and bead positions and velocities
    bit for bit (both parse the same text), fluid positions up to the wrap
    into the box (1e-13), the grid shift the reference reads (its mpcd.dat
    holds the address of the shift array, not the shift: both read 0);
  * continue like the reference on the same draws: 1e-10 in positions after
    two MPC steps of 50 MD substeps (the tolerance of the golden parity
    tests).
"""
import os
import shutil

import numpy as np
import pytest

import cilia_gpu as cg
from conftest import GOLDEN, golden

pytestmark = pytest.mark.gpu


def periodic_diff(a, b, L):
    d = a - b
    L = np.asarray(L, dtype=float)
    return d - np.round(d / L) * L


def ref_beads(g, tag):
    P, V = [], []
    for k in range(64):
        if f"{tag}_obj{k}_pos" in g:
            P.append(g[f"{tag}_obj{k}_pos"].reshape(-1, 3))
            V.append(g[f"{tag}_obj{k}_vel"].reshape(-1, 3))
    return np.concatenate(P), np.concatenate(V)


@pytest.mark.parametrize("arith", [cg.MD_DF, cg.MD_F64])
def test_resume_from_reference_checkpoints(tmp_path, monkeypatch, arith):
    g = golden("resume10")
    for key in g:
        if key.startswith("file_"):
            (tmp_path / key[5:]).write_bytes(g[key].tobytes())
    shutil.copy(os.path.join(GOLDEN, "cases", "clami10.cfg"), tmp_path / "clami10.cfg")
    monkeypatch.chdir(tmp_path)
    seed, steps, ststep = g["params"]
    s = cg.Sim("clami10.cfg", is_text=False, precision=cg.MPCD_FP64, ststep=float(ststep), seed=int(seed),
               create_fluid=True, read_files=True, md_arith=arith)
    e = s.engine
    L = (10, 10, 10)
    assert np.abs(e.shift - g["shift_0"]).max() < 1e-20
    p, v = e.fluid()
    assert p.shape == g["step0_fluid_pos"].shape
    assert np.abs(periodic_diff(p, g["step0_fluid_pos"], L)).max() < 1e-13
    assert np.array_equal(v, g["step0_fluid_vel"])
    bp, bv = s.beads()
    rp, rv = ref_beads(g, "step0")
    assert np.array_equal(bp, rp) and np.array_equal(bv, rv)
    for k in range(1, int(steps) + 1):
        s.next_tstep(g[f"shift_{k}"], g[f"gamma_{k}"], g[f"axis_{k}"])
    tag = f"step{int(steps)}"
    p, v = e.fluid()
    assert np.abs(periodic_diff(p, g[f"{tag}_fluid_pos"], L)).max() < 1e-10
    assert np.abs(v - g[f"{tag}_fluid_vel"]).max() < 1e-9
    bp, bv = s.beads()
    rp, rv = ref_beads(g, tag)
    assert np.abs(bp - rp).max() < 1e-10
    assert np.abs(bv - rv).max() < 1e-8
    assert abs(e.time - g[f"{tag}_meta"][0]) < 1e-12
    s.close()
