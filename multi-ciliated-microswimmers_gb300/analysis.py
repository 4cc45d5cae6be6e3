"""Swimmer analysis of the reference's output files, restated in numpy.

The reference analyses a run with pandas (sr/volvox/io.py, sr/volvox/process.py);
pandas is not a dependency here, so the same quantities are computed on plain
arrays, each function citing the reference lines it follows:

* `load_san`   - `<name>.san` rows of Clami::writedata (src/clami.cpp:208-284;
                 reader sr/volvox/io.py:58-82): time, centre of mass, its
                 velocity, the body frame n, b, p (sphere beads 1, 32, 137
                 minus bead 0) and the dissipated power.
* `load_xyz`   - `<name>.xyz` frames (sr/volvox/io.py:4-55).
* `rotation_rates` - body-frame rotation rates (sr/volvox/process.py:3-20).
* `analyze`    - the run's summary (sr/volvox/process.py:32-76).

Columns are returned as a dict of 1-D float arrays keyed by the reference's
column names.  Statistics skip NaN and standard deviations use one degree of
freedom less, as pandas' `mean`, `std`, `max` and `sum` do (an arccos of a dot
product that rounds above 1 is NaN in both).
"""
from __future__ import annotations

import numpy as np

SAN_COLUMNS = ["time", "x", "y", "z", "vx", "vy", "vz", "nx", "ny", "nz", "bx", "by", "bz", "px", "py", "pz",
               "power"]
# the first version of the file (sr/volvox/io.py:67-70)
SAN_COLUMNS_V1 = ["time", "x", "y", "z", "vx", "vy", "vz", "nx", "ny", "nz", "power"]
# a version with the kinetic energy after the velocity (sr/volvox/io.py:58-62)
SAN_COLUMNS_EKIN = ["time", "x", "y", "z", "vx", "vy", "vz", "ekin", "nx", "ny", "nz", "bx", "by", "bz", "px",
                    "py", "pz", "power"]


def load_san(path) -> dict:
    """Rows of a `.san` file as {column: array} (sr/volvox/io.py:58-82): 17
    columns as Clami::writedata writes them, 11 of the first version, or 18
    with the kinetic energy; columns a version lacks are NaN."""
    rows = np.atleast_2d(np.loadtxt(path, dtype=float))
    ncol = rows.shape[1]
    names = {17: SAN_COLUMNS, 11: SAN_COLUMNS_V1, 18: SAN_COLUMNS_EKIN}.get(ncol)
    if names is None:
        raise ValueError(f"{path}: {ncol} columns, not a swimmer .san file")
    out = {name: rows[:, k] for k, name in enumerate(names)}
    for name in SAN_COLUMNS_EKIN:
        out.setdefault(name, np.full(rows.shape[0], np.nan))
    return out


def load_xyz(path):
    """Frames of a `.xyz` file (sr/volvox/io.py:4-55): a count line, a comment
    line ending in the time, then one `<type> x y z` line per bead.  Returns
    (times[T], positions[T, n, 3]); a frame with a wrong number of lines is
    filled with NaN, as the reference fills it with None."""
    times, frames = [], []
    with open(path) as fp:
        lines = [ln.split() for ln in fp]
    i = 0
    t_prev = None
    while i < len(lines):
        if len(lines[i]) != 1:
            i += 1
            continue
        n = int(lines[i][0])
        try:
            t = float(lines[i + 1][-1])
        except (IndexError, ValueError):
            t = 0.0 if t_prev is None else t_prev + 1.0
        body = []
        j = i + 2
        while j < len(lines) and len(lines[j]) != 1:
            body.append([float(v) for v in lines[j][1:4]])
            j += 1
        frame = np.asarray(body, dtype=float) if len(body) == n else np.full((n, 3), np.nan)
        times.append(t)
        frames.append(frame)
        t_prev = t
        i = j
    return np.asarray(times), np.asarray(frames)


def normalize(vec: np.ndarray) -> np.ndarray:
    """Rows scaled to unit length (sr/volvox/process.py:23-24)."""
    return vec / np.sqrt((vec ** 2).sum(axis=1))[:, None]


def orientation(data: dict):
    """The unit body frame N, B, P (sr/volvox/process.py:26-30)."""
    def col(a, b, c):
        return np.stack([data[a], data[b], data[c]], axis=1)

    return (normalize(col("nx", "ny", "nz")), normalize(col("bx", "by", "bz")),
            normalize(col("px", "py", "pz")))


def rotation_rates(e: np.ndarray, b: np.ndarray, p: np.ndarray, time_step: float, k: int = 1):
    """Body-frame rotation rates (sr/volvox/process.py:3-20): over each of the
    k interleaved subsequences (rows l, l + k, ...; the last len % k rows
    dropped so that all have the same length) with numerical derivatives of
    spacing k * time_step, Omega_n = (p x dp/dt) . e, Omega_b = (p x dp/dt) .
    b and Omega_p = (e x de/dt) . p; the values are returned in row order.
    Returns (Omega_n, Omega_b, Omega_p), each of length len(e) - len(e) % k."""
    n = len(e)
    m = n - (n % k)
    on, ob, op = np.empty(m), np.empty(m), np.empty(m)
    for l in range(k):
        idx = np.arange(l, m, k)
        es, bs, ps = e[idx], b[idx], p[idx]
        ie = np.cross(es, np.gradient(es, time_step * k, axis=0))
        ip = np.cross(ps, np.gradient(ps, time_step * k, axis=0))
        on[idx] = np.sum(ip * es, axis=1)
        ob[idx] = np.sum(ip * bs, axis=1)
        op[idx] = np.sum(ie * ps, axis=1)
    return on, ob, op


def analyze(data: dict, eq_time: float = 500.0, k: int = 240, expect_tstep: float | None = 2.5):
    """The summary of a run (sr/volvox/process.py:32-76) from the rows at or
    after eq_time: the body axis' angle to its first direction (phi), the
    centre-of-mass velocity, the speed along the body axis, the rotation rates
    over k-row strides, |v| and the dissipated power.  The reference checks
    that rows are 2.5 time units apart (its output interval); expect_tstep=None
    skips the check.  As in the reference, the v_abs_y/z entries are taken
    from v_x.  Returns (results, N, V) with N the unit body axis and V the
    velocity rows after eq_time."""
    t = data["time"]
    tstep = float(np.mean(np.diff(t)))
    if expect_tstep is not None:
        assert tstep == expect_tstep, f"rows {tstep} time units apart, expected {expect_tstep}"
    sel = t >= eq_time
    sub = {key: v[sel] for key, v in data.items()}
    N, B, P = orientation(sub)
    mean, std = np.nanmean, (lambda x: np.nanstd(x, ddof=1))
    res = {}
    with np.errstate(invalid="ignore"):
        phi = np.arccos((N * N[0]).sum(axis=1))
    res["phi_mean"], res["phi_std"], res["phi_max"] = mean(phi), std(phi), np.nanmax(phi)
    V = np.stack([sub["vx"], sub["vy"], sub["vz"]], axis=1)
    res["vx_m"], res["vy_m"], res["vz_m"] = mean(V[:, 0]), mean(V[:, 1]), mean(V[:, 2])
    ax = np.abs(V[:, 0])
    res["v_abs_x_m"] = res["v_abs_y_m"] = res["v_abs_z_m"] = mean(ax)
    res["v_abs_x_std"] = res["v_abs_y_std"] = res["v_abs_z_std"] = std(ax)
    vn = (N * V).sum(axis=1)
    res["v_normal_m"], res["v_normal_std"] = mean(vn), std(vn)
    on, ob, op = rotation_rates(N, B, P, tstep, k)
    res["Omega_n_mean"], res["Omega_n_std"] = mean(on), std(on)
    res["Omega_b_mean"], res["Omega_b_std"] = mean(ob), std(ob)
    res["Omega_p_mean"], res["Omega_p_std"] = mean(op), std(op)
    ek = np.sqrt((V * V).sum(axis=1))
    res["e_kin_m"], res["e_kin_std"] = mean(ek), std(ek)
    pw = sub["power"]
    res["power_total"], res["power_mean"], res["power_std"] = np.nansum(pw), mean(pw), std(pw)
    return res, N, V
