"""mpcd_fluid_step_noalloc: the fluid step for callers that cannot allocate
device memory (code living inside another runtime's memory pool, or a plug-in
handed only pointers and a stream).  This test acts as such a caller: the
particle buffers come from torch's allocator and the call runs on torch's
stream.  Two calls in a row are checked against the engine's regular
split-precision step (mpcd_set_fluid + mpcd_step) on the same particles,
shifts and generator counters.

Both paths run the same kernels; they differ only in the order of the float
atomic additions into the cell sums, so the results agree to float rounding:
at least 99.9 % of the particles within 1e-4 in position and velocity, and
the dissipated energy within 1e-4 relative (the tolerances of the split
precision tests).  Runs alone in a fresh process as well as after the rest of
the suite (the static scratch keeps nothing a call depends on).
"""
import ctypes

import numpy as np
import pytest

import cilia_gpu as cg

pytestmark = pytest.mark.gpu


def pack_split(pos, vel, L):
    """Host arrays -> the split layout, rounding as mpcd_set_fluid does."""
    n = pos.shape[0]
    P = np.zeros((n, 4), dtype=np.float32)
    cells = np.zeros((n, 3), dtype=np.int64)
    for q in range(3):
        x = pos[:, q]
        xw = x - np.floor(x / L[q]) * L[q]
        xw = np.where(xw >= L[q], xw - L[q], xw)
        xw = np.where(xw < 0, xw + L[q], xw)
        fi = np.floor(xw)
        i = fi.astype(np.int64)
        o = xw - fi
        i = np.where(i >= L[q], i - L[q], i)
        wrap = o >= 1.0
        o = np.where(wrap, 0.0, o)
        i = np.where(wrap, (i + 1) % L[q], i)
        f = o.astype(np.float32)
        up = f >= np.float32(1.0)
        f = np.where(up, np.float32(0.0), f)
        i = np.where(up, (i + 1) % L[q], i)
        P[:, q] = f
        cells[:, q] = i
    packed = (cells[:, 0] | (cells[:, 1] << 10) | (cells[:, 2] << 20)).astype(np.uint32)
    P[:, 3] = packed.view(np.float32)
    V = np.zeros((n, 4), dtype=np.float32)
    V[:, :3] = vel.astype(np.float32)
    return P, V


def unpack_split(P, V):
    c = P[:, 3].view(np.uint32).astype(np.int64)
    cells = np.stack([c & 1023, (c >> 10) & 1023, (c >> 20) & 1023], axis=1)
    return cells + P[:, :3].astype(np.float64), V[:, :3].astype(np.float64)


def periodic_diff(a, b, L):
    d = a - b
    L = np.asarray(L, dtype=float)
    return d - np.round(d / L) * L


def test_noalloc_step_matches_engine_on_two_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    L = (16, 16, 16)
    n = L[0] * L[1] * L[2] * 10
    rng = np.random.default_rng(11)
    pos = rng.uniform(0, 16, (n, 3))
    vel = rng.normal(size=(n, 3))
    vel -= vel.mean(axis=0)
    seed = 1234
    e = cg.Engine(L, tstep=0.1, ststep=0.002, precision=cg.MPCD_FP32, seed=seed)
    e.set_fluid(pos, vel)
    a_cur = np.ascontiguousarray(e.shift)
    P, V = pack_split(pos, vel, L)
    dP = torch.from_numpy(P).cuda()
    dV = torch.from_numpy(V).cuda()
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    sizes = (ctypes.c_int * 3)(*L)
    lib = cg.lib()
    diss_prev = 0.0
    for step in (1, 2):
        e.step()
        a_next = np.ascontiguousarray(e.shift)
        diss = ctypes.c_double(0.0)
        rc = lib.mpcd_fluid_step_noalloc(sizes, n, ctypes.c_void_p(dP.data_ptr()), ctypes.c_void_p(dV.data_ptr()),
                                         0.1, a_cur.ctypes.data_as(cg._DP), a_next.ctypes.data_as(cg._DP),
                                         seed, step, ctypes.byref(diss), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, rc  # MPCD_OK
        pe, ve = e.fluid()
        ps, vs = unpack_split(dP.cpu().numpy(), dV.cpu().numpy())
        dp = np.abs(periodic_diff(ps, pe, L)).max(axis=1)
        dv = np.abs(vs - ve).max(axis=1)
        assert np.mean(dp < 1e-4) > 0.999, (step, np.sort(dp)[-5:])
        assert np.mean(dv < 1e-4) > 0.999, (step, np.sort(dv)[-5:])
        d_engine = e.observables()["diss_energy"] - diss_prev
        diss_prev += d_engine
        assert abs(diss.value - d_engine) <= 1e-4 * max(1.0, abs(d_engine)), (step, diss.value, d_engine)
        a_cur = a_next


def test_noalloc_rejects_boxes_beyond_the_static_scratch():
    lib = cg.lib()
    sizes = (ctypes.c_int * 3)(64, 64, 64)  # 262144 cells > the 65536-cell scratch
    a = np.full(3, 0.5)
    rc = lib.mpcd_fluid_step_noalloc(sizes, 0, None, None, 0.1, a.ctypes.data_as(cg._DP), a.ctypes.data_as(cg._DP),
                                     1, 1, None, None)
    assert rc == 1  # MPCD_EINVAL


def test_noalloc_steps_keep_the_oracle_statistics():
    """Twenty allocation-free steps of a 16^3 fluid created by the C oracle,
    beside twenty free-running steps of the oracle itself from the same
    state (different generators, so compared as statistics): total momentum
    conserved by both (float32 sums: 1e-5 per particle), and kT of both
    within 2 % of kT = 1 and of each other (the thermostat holds every cell at
    kT = 1; 40,960 particles fluctuate by about 0.4 %)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from oracle import OracleSim

    L = (16, 16, 16)
    o = OracleSim(L, tstep=0.1, ststep=0.002, seed=17)
    o.init_shift()
    o.fluid_create()
    o.init_bins()
    pos, vel = o.fluid()
    n = pos.shape[0]
    P0 = vel.sum(axis=0) / n
    P, V = pack_split(pos, vel, L)
    dP = torch.from_numpy(P).cuda()
    dV = torch.from_numpy(V).cuda()
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    sizes = (ctypes.c_int * 3)(*L)
    lib = cg.lib()
    rng = np.random.default_rng(4)
    a_cur = np.ascontiguousarray(o.shift)
    for step in range(1, 21):
        a_next = rng.uniform(0.0, 1.0, 3)
        rc = lib.mpcd_fluid_step_noalloc(sizes, n, ctypes.c_void_p(dP.data_ptr()), ctypes.c_void_p(dV.data_ptr()),
                                         0.1, a_cur.ctypes.data_as(cg._DP), a_next.ctypes.data_as(cg._DP),
                                         99, step, None, ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, (step, rc)
        a_cur = a_next
        o.step()
    _, vs = unpack_split(dP.cpu().numpy(), dV.cpu().numpy())
    _, vo = o.fluid()
    kt_gpu = float((vs ** 2).sum() / (3 * n))
    kt_orc = float((vo ** 2).sum() / (3 * n))
    assert np.abs(vs.sum(axis=0) / n - P0).max() < 1e-5
    assert np.abs(vo.sum(axis=0) / n - P0).max() < 1e-9
    assert abs(kt_gpu - 1.0) < 0.02 and abs(kt_orc - 1.0) < 0.02, (kt_gpu, kt_orc)
    assert abs(kt_gpu - kt_orc) < 0.02, (kt_gpu, kt_orc)


def test_noalloc_rejects_particles_outside_the_layout():
    """A caller-packed particle whose cell index lies beyond its box edge is
    rejected before any kernel indexes the scratch with it (the box is so
    small that even an unchecked index would stay inside the scratch array);
    the particles are left as they were."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    L = (4, 4, 4)
    rng = np.random.default_rng(8)
    n = 640
    P, V = pack_split(rng.uniform(0, 4, (n, 3)), rng.normal(size=(n, 3)), L)
    bad = P.copy()
    cp = np.uint32(5 | (1 << 10) | (2 << 20))  # ix = 5 in a box of edge 4
    bad[17, 3] = np.array([cp], dtype=np.uint32).view(np.float32)[0]
    dP = torch.from_numpy(bad).cuda()
    dV = torch.from_numpy(V).cuda()
    torch.cuda.synchronize()
    sizes = (ctypes.c_int * 3)(*L)
    a = np.full(3, 0.25)
    rc = cg.lib().mpcd_fluid_step_noalloc(sizes, n, ctypes.c_void_p(dP.data_ptr()), ctypes.c_void_p(dV.data_ptr()),
                                          0.1, a.ctypes.data_as(cg._DP), a.ctypes.data_as(cg._DP), 1, 1, None, None)
    assert rc == 4  # MPCD_EDEVICE
    assert np.array_equal(dP.cpu().numpy().view(np.uint32), bad.view(np.uint32))
    assert np.array_equal(dV.cpu().numpy(), V)
    bad2 = P.copy()
    bad2[3, 1] = np.float32(1.0)  # an offset outside [0, 1)
    dP = torch.from_numpy(bad2).cuda()
    torch.cuda.synchronize()
    rc = cg.lib().mpcd_fluid_step_noalloc(sizes, n, ctypes.c_void_p(dP.data_ptr()), ctypes.c_void_p(dV.data_ptr()),
                                          0.1, a.ctypes.data_as(cg._DP), a.ctypes.data_as(cg._DP), 1, 1, None, None)
    assert rc == 4
