import math

import numpy as np
import pytest

import simcfg
from conftest import GOLDEN


@pytest.mark.parametrize("case", ["fluid4", "clami10", "objects8"])
def test_roundtrip(case):
    cfg = simcfg.load(f"{GOLDEN}/cases/{case}.cfg")
    again = simcfg.parse(simcfg.dumps(cfg))
    assert again == cfg


def test_parse_syntax():
    txt = '''# comment
    a = 1; b : 2.5e1, c = "x" "y"; // tail
    /* block */ g = { h = [1, 2, 3]; l = ( {x = true;}, "s" ); };
    big = 0x10L;'''
    cfg = simcfg.parse(txt)
    assert cfg["a"] == 1 and cfg["b"] == 25.0 and cfg["c"] == "xy"
    assert cfg["g"]["h"] == [1, 2, 3] and cfg["g"]["l"][0]["x"] is True
    assert cfg["big"] == 16
    with pytest.raises(simcfg.ParseError):
        simcfg.parse("a = ;")
    with pytest.raises(simcfg.ParseError):
        simcfg.parse("a = 1; a = 2;")


def test_fibonacci_clami_geometry():
    o = simcfg.fibonacci_clami(100, radius=8.0, center=(32, 32, 32), seed=3)
    assert len(o["y_thetas"]) == 100 and len(o["start_delays"]) == 100
    r = 8.0 - 1.5
    pts = []
    for ty, tx in zip(o["y_thetas"], o["theta_offset"]):
        ty = math.radians(ty)
        pts.append((r * math.sin(ty), -r * math.cos(ty) * math.sin(tx), r * math.cos(tx) * math.cos(ty)))
    pts = np.array(pts)
    assert np.allclose(np.linalg.norm(pts, axis=1), r)
    d = np.linalg.norm(pts[:, None] - pts[None], axis=2) + np.eye(100) * 1e9
    assert d.min() > 1.0  # roughly uniform spacing on the sphere
    assert all(0 <= x < 100.0 for x in o["start_delays"])
