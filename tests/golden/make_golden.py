"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs oracle/_ref/ref_harness (the reference's own translation units plus a
harness; build it with `make -C oracle ref`) on the configurations in
tests/golden/cases/ and packs its outputs into compressed .npz files:

  <case>.npz   step0_* initial state, gamma_k / axis_k (per-cell Gamma variate
               and rotation axis the reference drew in step k), shift_k (grid
               shift after step k), stepK_* dumped states, replay_ok; the
               walls case also virt_k (virtual-particle momentum per cell).
  mt.npz       MT19937 outputs of the reference's MTRand for a few seeds and
               rgamma(Nc) samples (src/libcilia/mpcd.cpp:13-43).
  resume10.npz the checkpoint files a clami10 run leaves (the reference's own
               writers) and a second run resumed from them (run_resume).
  writers10.npz the .san / .xyz / mpcd.san text of the clami10 run (run_writers).

Usage: python tests/golden/make_golden.py   (needs the reference sources)
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(REPO, "oracle", "_ref", "ref_harness")
# the same harness built with -DNOSLIP -DFLUID_FLOW_G=0.02 (walls along z, body force along x)
HARNESS_WALLS = os.path.join(REPO, "oracle", "_ref", "ref_harness_walls")

# case name: (seed, steps, ststep, dump list, harness)
CASES = {
    "fluid4": (11, 5, 0.002, "1,5", HARNESS),
    "fluid8": (7, 3, 0.002, "3", HARNESS),
    "clami10": (3, 4, 0.002, "4", HARNESS),
    "objects8": (3, 4, 0.002, "4", HARNESS),
    "walls8": (9, 5, 0.002, "1,5", HARNESS_WALLS),
}


def run_case(name, seed, steps, ststep, dumps, harness=HARNESS):
    cfg = os.path.join(HERE, "cases", name + ".cfg")
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "out")
        subprocess.run([harness, "run", cfg, out, str(seed), str(steps), repr(ststep), dumps],
                       check=True, stdout=subprocess.DEVNULL)
        arrays = {}
        with open(os.path.join(out, "index.txt")) as f:
            for line in f:
                parts = line.split()
                shape = tuple(int(x) for x in parts[1:])
                arrays[parts[0]] = np.fromfile(os.path.join(out, parts[0] + ".f64")).reshape(shape)
    arrays["params"] = np.array([seed, steps, ststep], dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    return arrays


def run_resume(name="clami10", seed=3, steps1=2, steps2=2, ststep=0.002):
    """resume<case>.npz: a run of `steps1` steps whose destructor leaves the
    reference's checkpoint files (fluid_n.dat, mpcd.dat, <object>.dat), then a
    second run started in the same directory, which loads them (Simulation's
    constructor: Fluid::FluidFromFile, MDObject::open_datfile, the MPCD
    constructor's mpcd.dat) and runs `steps2` recorded steps.  Stored: the
    checkpoint files as written (file_<name>, bytes), and the second run's
    step0 (the loaded state), draws and final state."""
    cfg = os.path.join(HERE, "cases", name + ".cfg")
    arrays = {}
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "out")
        subprocess.run([HARNESS, "run", cfg, out, str(seed), str(steps1), repr(ststep), ""],
                       check=True, stdout=subprocess.DEVNULL)
        for fn in sorted(os.listdir(out)):
            if fn.endswith(".dat"):
                with open(os.path.join(out, fn), "rb") as f:
                    arrays["file_" + fn] = np.frombuffer(f.read(), dtype=np.uint8)
        for fn in os.listdir(out):  # the second run writes its own outputs
            if not fn.endswith(".dat"):
                os.remove(os.path.join(out, fn))
        subprocess.run([HARNESS, "run", cfg, out, str(seed), str(steps2), repr(ststep), str(steps2)],
                       check=True, stdout=subprocess.DEVNULL)
        with open(os.path.join(out, "index.txt")) as f:
            for line in f:
                parts = line.split()
                shape = tuple(int(x) for x in parts[1:])
                arrays[parts[0]] = np.fromfile(os.path.join(out, parts[0] + ".f64")).reshape(shape)
    arrays["params"] = np.array([seed, steps2, ststep], dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "resume" + name.replace("clami", "") + ".npz"), **arrays)
    return arrays


def run_writers(name="clami10", seed=3, steps=4, ststep=0.002, writes="2,4"):
    """writers<case>.npz: the text the reference's writers produce on the run
    of tests/golden/<case>.npz (same seed, steps and MD step): the Clami's
    <name>.san and <name>.xyz (Clami::writedata) and mpcd.san (MPCD::debug,
    its first row from Simulation's constructor), written after the steps of
    `writes` as Simulation::run writes after a measure interval."""
    cfg = os.path.join(HERE, "cases", name + ".cfg")
    arrays = {}
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "out")
        subprocess.run([HARNESS, "run", cfg, out, str(seed), str(steps), repr(ststep), "", writes],
                       check=True, stdout=subprocess.DEVNULL)
        for fn in sorted(os.listdir(out)):
            if fn.endswith((".san", ".xyz")):
                with open(os.path.join(out, fn), "rb") as f:
                    arrays["file_" + fn] = np.frombuffer(f.read(), dtype=np.uint8)
        arrays[f"shift_{steps}"] = np.fromfile(os.path.join(out, f"shift_{steps}.f64"))
    arrays["params"] = np.array([seed, steps, ststep], dtype=np.float64)
    arrays["writes"] = np.array([int(x) for x in writes.split(",")], dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "writers" + name.replace("clami", "") + ".npz"), **arrays)
    return arrays


def run_mt():
    out = {}
    for seed in (1, 5489, 4357):
        txt = subprocess.run([HARNESS, "kat", str(seed), "2000"], check=True, capture_output=True, text=True).stdout
        out[f"kat_{seed}"] = np.array([int(x) for x in txt.split()], dtype=np.uint64)
    for nc in (2, 5, 10, 30):
        txt = subprocess.run([HARNESS, "gamma", "42", str(nc), "500"], check=True, capture_output=True, text=True).stdout
        out[f"gamma42_{nc}"] = np.array([float(x) for x in txt.split()])
    np.savez_compressed(os.path.join(HERE, "mt.npz"), **out)


def main():
    """python make_golden.py [case ...]: every case (and mt.npz), or the named ones."""
    if not os.path.exists(HARNESS):
        sys.exit("build the reference harness first: make -C oracle ref")
    names = sys.argv[1:] or list(CASES) + ["mt", "resume", "writers"]
    for name in names:
        if name == "mt":
            run_mt()
            print("mt.npz written")
            continue
        if name == "writers":
            a = run_writers()
            print("writers10.npz arrays:", len(a))
            continue
        if name == "resume":
            a = run_resume()
            print("resume10.npz arrays:", len(a), "replay_ok:", a["replay_ok"][0])
            continue
        seed, steps, ststep, dumps, harness = CASES[name]
        a = run_case(name, seed, steps, ststep, dumps, harness)
        print(name, "arrays:", len(a), "replay_ok:", a["replay_ok"][0])


if __name__ == "__main__":
    main()
