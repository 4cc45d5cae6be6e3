"""The numpy restatement of the reference's swimmer analysis
(sr/volvox/io.py, sr/volvox/process.py) on inputs whose answers are known in
closed form: a body frame turning at a constant rate about one of its axes
gives that rate exactly times sin(w dt)/(w dt) for derivatives over dt (the
chord of the turn), and zero about the other two axes."""
import numpy as np
import pytest

import analysis


def frame_about_p(t, w):
    c, s = np.cos(w * t), np.sin(w * t)
    z = np.zeros_like(t)
    n = np.stack([c, s, z], axis=1)
    b = np.stack([-s, c, z], axis=1)
    p = np.stack([z, z, np.ones_like(t)], axis=1)
    return n, b, p


def test_rotation_about_p_and_about_n():
    t = np.arange(0.0, 300.0, 0.5)
    w = 0.02
    n, b, p = frame_about_p(t, w)
    on, ob, op = analysis.rotation_rates(n, b, p, 0.5, 1)
    chord = w * np.sin(w * 0.5) / (w * 0.5)
    assert np.allclose(op, chord, rtol=0, atol=1e-12)
    assert np.abs(on).max() < 1e-15 and np.abs(ob).max() < 1e-15
    # the same turn seen with n as the axis: p and b turn about n
    on2, ob2, op2 = analysis.rotation_rates(p, n, b, 0.5, 1)
    assert np.allclose(on2, chord, atol=1e-12) and np.abs(op2).max() < 1e-15


def test_strided_subsequences_in_row_order():
    rng = np.random.default_rng(1)
    m, k = 103, 4
    e, b, p = (analysis.normalize(rng.normal(size=(m, 3))) for _ in range(3))
    on, ob, op = analysis.rotation_rates(e, b, p, 2.5, k)
    assert len(on) == m - m % k
    for l in range(k):  # each subsequence on its own, spacing k * dt
        idx = np.arange(l, m - m % k, k)
        ref_on, ref_ob, ref_op = analysis.rotation_rates(e[idx], b[idx], p[idx], 2.5 * k, 1)
        assert np.array_equal(on[idx], ref_on) and np.array_equal(ob[idx], ref_ob) and np.array_equal(op[idx], ref_op)


def write_san(path, rows):
    np.savetxt(path, rows, fmt="%.17g")


def test_analyze_a_swimmer_turning_about_its_p_axis(tmp_path):
    dt, w, v0 = 2.5, 1e-4, 0.01
    t = np.arange(0.0, 3750.0, dt)
    n, b, p = frame_about_p(t, w)
    v = v0 * n  # swims along its body axis
    x = np.cumsum(v, axis=0) * dt
    rng = np.random.default_rng(3)
    power = rng.uniform(0.5, 1.5, len(t))
    rows = np.column_stack([t, x, v, 2.0 * n, 3.0 * b, 0.5 * p, power])  # unnormalised frame, as written
    write_san(tmp_path / "volvox.san", rows)
    data = analysis.load_san(tmp_path / "volvox.san")
    assert set(analysis.SAN_COLUMNS) <= set(data) and np.isnan(data["ekin"]).all()
    res, N, V = analysis.analyze(data, eq_time=500.0)
    sel = t >= 500.0
    ts = t[sel] - t[sel][0]
    assert res["phi_max"] == pytest.approx(w * ts[-1], rel=1e-9)
    assert res["phi_mean"] == pytest.approx(np.mean(w * ts), rel=1e-6)
    assert res["v_normal_m"] == pytest.approx(v0, rel=1e-12) and res["v_normal_std"] < 1e-15
    assert res["e_kin_m"] == pytest.approx(v0, rel=1e-12)
    assert res["vx_m"] == pytest.approx(np.mean(v[sel, 0]), rel=1e-12)
    assert res["v_abs_y_m"] == res["v_abs_x_m"]  # the reference takes both from v_x
    h = dt * 240
    assert res["Omega_p_mean"] == pytest.approx(w * np.sin(w * h) / (w * h), rel=1e-9)
    assert abs(res["Omega_n_mean"]) < 1e-15 and abs(res["Omega_b_mean"]) < 1e-15
    assert res["power_total"] == pytest.approx(power[sel].sum(), rel=1e-12)
    assert res["power_std"] == pytest.approx(np.std(power[sel], ddof=1), rel=1e-12)
    assert N.shape == (sel.sum(), 3) and V.shape == (sel.sum(), 3)
    with pytest.raises(AssertionError):
        analysis.analyze({**data, "time": data["time"] * 2.0}, eq_time=500.0)
    analysis.analyze({**data, "time": data["time"] * 2.0}, eq_time=500.0, expect_tstep=None)


def test_first_version_san_and_xyz_frames(tmp_path):
    rows = np.column_stack([np.arange(4.0), np.ones((4, 9)), np.full(4, 0.25)])
    write_san(tmp_path / "v1.san", rows)
    d = analysis.load_san(tmp_path / "v1.san")
    assert np.array_equal(d["power"], np.full(4, 0.25)) and np.isnan(d["bx"]).all()
    with open(tmp_path / "a.xyz", "w") as f:
        f.write("2\nrods: 1.5\nH 0 1 2\nO 3 4 5\n2\nrods: 2.5\nH 6 7 8\n2\nrods: 3.5\nH 1 1 1\nO 2 2 2\n")
    times, frames = analysis.load_xyz(tmp_path / "a.xyz")
    assert np.array_equal(times, [1.5, 2.5, 3.5]) and frames.shape == (3, 2, 3)
    assert np.array_equal(frames[0], [[0, 1, 2], [3, 4, 5]]) and np.isnan(frames[1]).all()
