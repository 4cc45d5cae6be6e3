"""The host object model (the reference's Simulation constructor, rebuilt in
C++ above the engine) against the reference's own initial state, on the CPU:
cilia_cfg_host_state builds a sim.cfg's system without a GPU.  The golden
fixtures were written by the reference itself (oracle/_ref/ref_harness)."""
import numpy as np
import pytest

import cilia_gpu as cg
from conftest import GOLDEN, golden


def ref_beads(g, tag):
    P, V = [], []
    for k in range(64):
        if f"{tag}_obj{k}_pos" in g:
            P.append(g[f"{tag}_obj{k}_pos"].reshape(-1, 3))
            V.append(g[f"{tag}_obj{k}_vel"].reshape(-1, 3))
    return (np.concatenate(P), np.concatenate(V)) if P else (np.zeros((0, 3)), np.zeros((0, 3)))


@pytest.mark.parametrize("case", ["clami10", "objects8"])
def test_geometry_matches_reference(case):
    """Sphere::create / create_neillist (the refined icosahedron), Cilia::create
    and the Clami's cilia placement give the reference's bead positions and
    velocities (src/sphere.cpp:136-285, src/cilia.cpp:275-325, src/clami.cpp:120-198)."""
    g = golden(case)
    text = open(f"{GOLDEN}/cases/{case}.cfg").read()
    st = cg.cfg_host_state(text, seed=int(g["params"][0]), create_fluid=False)
    rp, rv = ref_beads(g, "step0")
    assert st["bead_pos"].shape == rp.shape and len(rp) > 0
    assert np.abs(st["bead_pos"] - rp).max() < 1e-13
    assert np.abs(st["bead_vel"] - rv).max() < 1e-13
    assert st["nsprings"] > 0 and st["fluid_pos"].shape == (0, 3)


@pytest.mark.parametrize("case", ["fluid4", "fluid8", "clami10", "objects8"])
def test_initial_shift_and_fluid_match_reference(case):
    """MPCD's grid shift and Fluid::create (src/libcilia/mpcd.cpp:86-97,
    src/libcilia/fluid.cpp:55-98) from the same MT19937 stream: shift and
    positions bit for bit, velocities to 1e-14 (the reference is compiled with
    -ffast-math, so its Box-Muller transform and the mean subtraction may round
    differently in the last bit)."""
    g = golden(case)
    text = open(f"{GOLDEN}/cases/{case}.cfg").read()
    st = cg.cfg_host_state(text, seed=int(g["params"][0]), create_fluid=True)
    assert np.array_equal(st["shift"], g["shift_0"])
    assert st["fluid_pos"].shape == g["step0_fluid_pos"].shape
    assert np.array_equal(st["fluid_pos"], g["step0_fluid_pos"])
    assert np.abs(st["fluid_vel"] - g["step0_fluid_vel"]).max() < 1e-14
    assert np.abs(st["fluid_vel"].mean(axis=0)).max() < 1e-12


def test_cfg_errors_come_back_as_messages():
    with pytest.raises(cg.MpcdError, match="md_objects|No "):
        cg.cfg_host_state("sizex = 8; sizey = 8; sizez = 8;", create_fluid=False)
    with pytest.raises(cg.MpcdError, match="Parse error"):
        cg.cfg_host_state("sizex = ;", create_fluid=False)


def test_libconfig_syntax_variants_build_the_same_system():
    """The cfg reader takes libconfig's syntax variants as the reference's
    libconfig++ does: ':' for '=', '//' and '/* */' comments, exponents, a
    trailing comma-free list, whitespace anywhere; the system is the same."""
    text = open(f"{GOLDEN}/cases/objects8.cfg").read()
    v = text.replace("springconstant = 2000.0;", "springconstant : 2.0e3; // the sphere's springs")
    v = v.replace("rodlength = 5;", "/* five\n   sections */ rodlength=5 ;")
    v = v.replace("position = [ 5.0, 5.0, 3.0 ];", "position:[5.0,5.0,\n 3.0];")
    assert v != text
    a = cg.cfg_host_state(text, seed=3, create_fluid=True)
    b = cg.cfg_host_state(v, seed=3, create_fluid=True)
    for k in ("shift", "fluid_pos", "fluid_vel", "bead_pos", "bead_vel"):
        assert np.array_equal(a[k], b[k]), k
    assert a["nsprings"] == b["nsprings"]
