"""ctypes binding of libmpcd_gpu.so (include/mpcd_gpu.h, include/cilia_host.h,
include/mpcd_batch.h).

`Engine` wraps one mpcd_engine (a box of MPCD fluid plus MD beads on the GPU);
`Sim` wraps one cilia_sim (the reference's Simulation built from a sim.cfg);
`Batch` wraps one mpcd_batch (many independent boxes advanced together).
There is no CPU fallback: if the library or a GPU is missing, construction
raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libmpcd_gpu.so")

MPCD_FP64, MPCD_FP32 = 0, 1
WALLS_NONE, WALLS_NOSLIP, WALLS_SLIP = 0, 1, 2
SPRING_CONST, SPRING_GUARDED, SPRING_BOND, SPRING_DIAG = 0, 1, 2, 3
CILIUM_BASIC, CILIUM_CONSTANT = 0, 1
K_CELL, K_FLUID, K_BEAD, K_MD, K_SORT = 0, 1, 2, 3, 4
# MD arithmetic (mpcd_params.md_split): auto, float64, split floats (cluster
# layout), double-float, float springs on the double-float grid layout,
# float64 and double-float with each spring pair evaluated once (pair kernel)
MD_AUTO, MD_F64, MD_SPLIT, MD_DF, MD_FLOAT, MD_PAIR, MD_PAIR_DF = -1, 0, 1, 2, 3, 4, 5
OBS_RING = 256  # observables tickets a handle keeps collectable (MPCD_OBS_RING)

_D = ctypes.c_double
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)


class MpcdParams(ctypes.Structure):
    _fields_ = [("sizes", ctypes.c_int * 3), ("tstep", _D), ("ststep", _D), ("precision", ctypes.c_int),
                ("walls", ctypes.c_int), ("gravity", _D), ("omega", _D), ("bead_mass", _D),
                ("seed", ctypes.c_ulonglong), ("device", ctypes.c_int), ("sort_interval", ctypes.c_int),
                ("md_split", ctypes.c_int)]


class MpcdInject(ctypes.Structure):
    _fields_ = [("shift_next", _DP), ("gamma", _DP), ("axis", _DP), ("virt", _DP)]


class MpcdObs(ctypes.Structure):
    _fields_ = [("momentum", _D * 3), ("n", _D), ("mass", _D), ("kT", _D), ("fluid_T", _D),
                ("diss_energy", _D), ("globalt", _D), ("energy_fluid", _D)]


class MpcdCilium(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("rodlength", ctypes.c_int), ("num_anker", ctypes.c_int),
                ("bead0", ctypes.c_int), ("bond_base", ctypes.c_int), ("beatstrength", _D), ("bending", _D),
                ("max_bend", _D), ("m_speed", _D), ("power_stroke_duration", _D),
                ("recovery_stroke_duration", _D), ("start", _D), ("midpnt", _D), ("tstroke", _D)]


class CiliaOptions(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("device", ctypes.c_int), ("seed", ctypes.c_ulonglong),
                ("ststep", _D), ("create_fluid", ctypes.c_int), ("read_files", ctypes.c_int),
                ("walls", ctypes.c_int), ("gravity", _D), ("bead_mass", _D), ("sort_interval", ctypes.c_int),
                ("md_arith", ctypes.c_int)]


class MpcdBatchParams(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("max_replicas", ctypes.c_int), ("max_particles", ctypes.c_long),
                ("max_cells", ctypes.c_long), ("max_slots", ctypes.c_long), ("max_springs", ctypes.c_long),
                ("max_halo", ctypes.c_long), ("max_cilia", ctypes.c_int), ("max_bonds", ctypes.c_long),
                ("md_lanes", ctypes.c_int), ("md_tile", ctypes.c_int), ("sort_interval", ctypes.c_int),
                ("sorts_per_graph", ctypes.c_int)]


class MpcdBatchTuning(ctypes.Structure):
    _fields_ = [("fluid_threads", ctypes.c_int), ("fluid_blocks", ctypes.c_int), ("cell_threads", ctypes.c_int),
                ("cell_blocks", ctypes.c_int), ("sort_interval", ctypes.c_int)]


class MpcdServerParams(ctypes.Structure):
    _fields_ = [("batch", MpcdBatchParams), ("budget_bytes", ctypes.c_longlong), ("chunk_steps", ctypes.c_int),
                ("keep_fluid", ctypes.c_int), ("lookahead", ctypes.c_int), ("prep_threads", ctypes.c_int),
                ("preempt_wait_s", _D)]


class MpcdRequestInfo(ctypes.Structure):
    _fields_ = [("id", ctypes.c_longlong), ("state", ctypes.c_int), ("steps", ctypes.c_longlong),
                ("t_submit", _D), ("t_admit", _D), ("t_done", _D), ("nfluid", ctypes.c_longlong),
                ("nbeads", ctypes.c_longlong), ("footprint", ctypes.c_longlong), ("obs", MpcdObs),
                ("err_bits", ctypes.c_uint), ("preemptions", ctypes.c_int)]


class MpcdServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_longlong), ("completed", ctypes.c_longlong), ("failed", ctypes.c_longlong),
                ("resident", ctypes.c_longlong), ("queued", ctypes.c_longlong), ("p50_s", _D), ("p99_s", _D),
                ("mean_s", _D), ("max_s", _D), ("particle_steps", _D), ("busy_s", _D), ("throughput", _D),
                ("peak_resident_bytes", ctypes.c_longlong), ("peak_resident", ctypes.c_int),
                ("gpu_launches", ctypes.c_longlong), ("preemptions", ctypes.c_longlong)]


REQ_QUEUED, REQ_RESIDENT, REQ_DONE, REQ_FAILED = 0, 1, 2, 3


class MpcdRigidSphere(ctypes.Structure):
    _fields_ = [("center", ctypes.c_double * 3), ("velocity", ctypes.c_double * 3), ("omega", ctypes.c_double * 3),
                ("radius", ctypes.c_double), ("mass", ctypes.c_double)]


class MpcdError(RuntimeError):
    pass


_lib = None


def lib():
    """Load libmpcd_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise MpcdError(f"{LIB_PATH} not built: run build.py (or __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        sig = {
            "mpcd_create": (ctypes.c_int, [ctypes.POINTER(MpcdParams), ctypes.POINTER(P)]),
            "mpcd_destroy": (ctypes.c_int, [P]),
            "mpcd_last_error": (ctypes.c_char_p, [P]),
            "mpcd_cell_count": (ctypes.c_long, [P]),
            "mpcd_set_fluid": (ctypes.c_int, [P, ctypes.c_long, _DP, _DP]),
            "mpcd_get_fluid": (ctypes.c_int, [P, ctypes.c_long, _DP, _DP]),
            "mpcd_fluid_count": (ctypes.c_long, [P]),
            "mpcd_set_shift": (ctypes.c_int, [P, _DP]),
            "mpcd_get_shift": (ctypes.c_int, [P, _DP]),
            "mpcd_set_time": (ctypes.c_int, [P, _D]),
            "mpcd_get_time": (ctypes.c_int, [P, _DP]),
            "mpcd_set_beads": (ctypes.c_int, [P, ctypes.c_long, _DP, _DP, _IP]),
            "mpcd_get_beads": (ctypes.c_int, [P, ctypes.c_long, _DP, _DP]),
            "mpcd_set_springs": (ctypes.c_int, [P, ctypes.c_long, _IP, _IP, _IP, _IP, _DP, _DP]),
            "mpcd_set_cilia": (ctypes.c_int, [P, ctypes.c_int, ctypes.POINTER(MpcdCilium), _DP, _DP]),
            "mpcd_get_cilia": (ctypes.c_int, [P, ctypes.c_int, _DP, _DP, _DP]),
            "mpcd_prepare": (ctypes.c_int, [P]),
            "mpcd_step": (ctypes.c_int, [P, ctypes.POINTER(MpcdInject)]),
            "mpcd_run": (ctypes.c_int, [P, ctypes.c_int]),
            "mpcd_observables": (ctypes.c_int, [P, ctypes.POINTER(MpcdObs)]),
            "mpcd_pin_host": (ctypes.c_int, [P, P, ctypes.c_size_t]),
            "mpcd_unpin_host": (ctypes.c_int, [P, P]),
            "mpcd_observables_async": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_longlong)]),
            "mpcd_observables_result": (ctypes.c_int, [P, ctypes.c_longlong, ctypes.POINTER(MpcdObs)]),
            "mpcd_reset_diss": (ctypes.c_int, [P]),
            "mpcd_sync": (ctypes.c_int, [P]),
            "mpcd_launch_count": (ctypes.c_longlong, [P]),
            "mpcd_timed_run": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, _DP]),
            "mpcd_set_profiling": (ctypes.c_int, [P, ctypes.c_int]),
            "mpcd_kernel_time": (ctypes.c_int, [P, ctypes.c_int, _DP, ctypes.POINTER(ctypes.c_longlong)]),
            "mpcd_md_layout": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_int)]),
            "mpcd_fluid_step_noalloc": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int), ctypes.c_long, P, P, _D, _DP, _DP,
                                                       ctypes.c_ulonglong, ctypes.c_ulonglong, _DP, P]),
            "mpcd_snapshot_size": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_longlong)]),
            "mpcd_snapshot": (ctypes.c_int, [P, ctypes.c_void_p, ctypes.c_longlong]),
            "mpcd_restore": (ctypes.c_int, [P, ctypes.c_void_p, ctypes.c_longlong]),
            "mpcd_set_rigid_spheres": (ctypes.c_int, [P, ctypes.c_int, ctypes.POINTER(MpcdRigidSphere)]),
            "mpcd_get_rigid_spheres": (ctypes.c_int, [P, ctypes.c_int, ctypes.POINTER(MpcdRigidSphere), _DP]),
            "mpcd_reset_rigid_sphere_forces": (ctypes.c_int, [P]),
            "mpcd_rigid_sphere_count": (ctypes.c_int, [P]),
            "mpcd_set_repelling": (ctypes.c_int, [P, _D]),
            "mpcd_collision_draws": (ctypes.c_int, [ctypes.c_int, ctypes.c_ulonglong, ctypes.c_ulonglong, ctypes.c_long,
                                                    _DP, _DP, ctypes.c_int]),
            "mpcd_batch_step_inject": (ctypes.c_int, [P, ctypes.c_int, ctypes.POINTER(MpcdInject)]),
            "mpcd_batch_create": (ctypes.c_int, [ctypes.POINTER(MpcdBatchParams), ctypes.POINTER(P)]),
            "mpcd_batch_destroy": (ctypes.c_int, [P]),
            "mpcd_batch_last_error": (ctypes.c_char_p, [P]),
            "mpcd_batch_add": (ctypes.c_int, [P, ctypes.POINTER(MpcdParams), _IP]),
            "mpcd_batch_add_engine": (ctypes.c_int, [P, P, _IP]),
            "mpcd_batch_set_fluid": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_long, _DP, _DP]),
            "mpcd_batch_set_shift": (ctypes.c_int, [P, ctypes.c_int, _DP]),
            "mpcd_batch_set_time": (ctypes.c_int, [P, ctypes.c_int, _D]),
            "mpcd_batch_set_beads": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_long, _DP, _DP, _IP]),
            "mpcd_batch_set_springs": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_long, _IP, _IP, _IP, _IP, _DP, _DP]),
            "mpcd_batch_set_cilia": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(MpcdCilium), _DP,
                                                    _DP]),
            "mpcd_batch_footprint": (ctypes.c_int, [P, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]),
            "mpcd_batch_estimate": (ctypes.c_longlong, [P, ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.c_long,
                                                        ctypes.c_int, ctypes.c_long]),
            "cilia_batch_add_cfg": (ctypes.c_int, [P, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(CiliaOptions),
                                                   _IP]),
            "mpcd_batch_admit": (ctypes.c_int, [P, ctypes.c_int]),
            "mpcd_batch_set_steps": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_longlong]),
            "mpcd_batch_run": (ctypes.c_int, [P, ctypes.c_int]),
            "mpcd_batch_timed_run": (ctypes.c_int, [P, ctypes.c_int, _DP]),
            "mpcd_batch_sync": (ctypes.c_int, [P]),
            "mpcd_batch_status": (ctypes.c_int, [P, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong),
                                                 ctypes.POINTER(ctypes.c_longlong), _DP,
                                                 ctypes.POINTER(ctypes.c_uint)]),
            "mpcd_batch_get_fluid": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_long, _DP, _DP]),
            "mpcd_batch_get_beads": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_long, _DP, _DP]),
            "mpcd_batch_get_shift": (ctypes.c_int, [P, ctypes.c_int, _DP]),
            "mpcd_batch_observables": (ctypes.c_int, [P, ctypes.c_int, ctypes.POINTER(MpcdObs)]),
            "mpcd_batch_remove": (ctypes.c_int, [P, ctypes.c_int]),
            "mpcd_batch_resident": (ctypes.c_int, [P]),
            "mpcd_batch_autotune": (ctypes.c_int, [P, ctypes.c_int, ctypes.POINTER(MpcdBatchTuning)]),
            "mpcd_batch_set_tuning": (ctypes.c_int, [P, ctypes.POINTER(MpcdBatchTuning)]),
            "mpcd_batch_get_tuning": (ctypes.c_int, [P, ctypes.POINTER(MpcdBatchTuning)]),
            "mpcd_batch_launch_count": (ctypes.c_longlong, [P]),
            "mpcd_batch_stage_times": (ctypes.c_int, [P, ctypes.c_int, _DP]),
            "mpcd_batch_set_md_layout": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int]),
            "mpcd_batch_get_md_layout": (ctypes.c_int, [P, _IP, _IP]),
            "mpcd_server_create": (ctypes.c_int, [ctypes.POINTER(MpcdServerParams), ctypes.POINTER(P)]),
            "mpcd_server_destroy": (ctypes.c_int, [P]),
            "mpcd_server_last_error": (ctypes.c_char_p, [P]),
            "mpcd_server_submit": (ctypes.c_int, [P, ctypes.c_char_p, ctypes.c_longlong, ctypes.c_ulonglong,
                                                  ctypes.POINTER(ctypes.c_longlong)]),
            "mpcd_server_info": (ctypes.c_int, [P, ctypes.c_longlong, ctypes.POINTER(MpcdRequestInfo)]),
            "mpcd_server_wait": (ctypes.c_int, [P, ctypes.c_longlong, _D, ctypes.POINTER(MpcdRequestInfo)]),
            "mpcd_server_drain": (ctypes.c_int, [P, _D]),
            "mpcd_server_result_beads": (ctypes.c_int, [P, ctypes.c_longlong, ctypes.c_long, _DP, _DP]),
            "mpcd_server_result_fluid": (ctypes.c_int, [P, ctypes.c_longlong, ctypes.c_long, _DP, _DP]),
            "mpcd_server_get_stats": (ctypes.c_int, [P, ctypes.POINTER(MpcdServerStats)]),
            "mpcd_server_request_error": (ctypes.c_char_p, [P, ctypes.c_longlong]),
            "mpcd_server_preempt": (ctypes.c_int, [P, ctypes.c_longlong]),
            "mpcd_batch_get_cilia": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_int, _DP, _DP, _DP]),
            "mpcd_batch_set_step_count": (ctypes.c_int, [P, ctypes.c_int, ctypes.c_longlong]),
            "cilia_sim_create": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(CiliaOptions),
                                                ctypes.POINTER(P)]),
            "cilia_sim_destroy": (ctypes.c_int, [P]),
            "cilia_sim_last_error": (ctypes.c_char_p, [P]),
            "cilia_sim_engine": (P, [P]),
            "cilia_sim_num_objects": (ctypes.c_int, [P]),
            "cilia_sim_object_info": (ctypes.c_int, [P, ctypes.c_int, _IP, ctypes.c_char_p, ctypes.c_int]),
            "cilia_sim_bead_count": (ctypes.c_long, [P]),
            "cilia_sim_next_tstep": (ctypes.c_int, [P, ctypes.POINTER(MpcdInject)]),
            "cilia_sim_run": (ctypes.c_int, [P]),
            "cilia_sim_save": (ctypes.c_int, [P]),
            "cilia_sim_writedata": (ctypes.c_int, [P, ctypes.c_int]),
            "cilia_sim_write_cfg": (ctypes.c_int, [P, ctypes.c_char_p]),
            "cilia_cfg_host_state": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(CiliaOptions),
                                                    ctypes.POINTER(ctypes.c_long), _DP, _DP, _DP, _DP, _DP]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def collision_draws(nc, n, *, seed=1, step=1, device=0, gamma=True, axis=True):
    """The device generator's per-cell draws of one step (mpcd_collision_draws):
    Gamma(3(nc-1)/2) variates and float64-path rotation axes of cells 0..n-1."""
    g = np.zeros(n) if gamma else None
    a = np.zeros((n, 3)) if axis else None
    rc = lib().mpcd_collision_draws(int(nc), int(seed), int(step), int(n), _dp(g), _dp(a), int(device))
    if rc:
        raise MpcdError(f"mpcd_collision_draws failed ({rc})")
    return g, a


def _dp(a):
    return None if a is None else a.ctypes.data_as(_DP)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class Engine:
    """One MPCD box with MD beads on the GPU (mpcd_engine)."""

    def __init__(self, L, *, tstep=0.1, ststep=0.001, precision=MPCD_FP64, walls=WALLS_NONE, gravity=0.0,
                 omega=0.0, bead_mass=5.0, seed=1, device=0, sort_interval=0, md_split=-1, _handle=None,
                 _owner=None):
        self._owner = _owner
        if _handle is not None:
            self._h = _handle
            self._owns = False
        else:
            if isinstance(L, int):
                L = (L, L, L)
            p = MpcdParams()
            p.sizes[:] = [int(x) for x in L]
            p.tstep, p.ststep, p.precision, p.walls = tstep, ststep, precision, walls
            p.gravity, p.omega, p.bead_mass, p.seed = gravity, omega, bead_mass, seed
            p.device, p.sort_interval, p.md_split = device, sort_interval, md_split
            h = ctypes.c_void_p()
            rc = lib().mpcd_create(ctypes.byref(p), ctypes.byref(h))
            if rc:
                raise MpcdError(f"mpcd_create failed with code {rc}")
            self._h = h
            self._owns = True

    def close(self):
        if getattr(self, "_owns", False) and self._h:
            lib().mpcd_destroy(self._h)
        self._h = None

    def __del__(self):
        self.close()

    def _ck(self, rc, what):
        if rc:
            msg = lib().mpcd_last_error(self._h)
            raise MpcdError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")

    @property
    def handle(self):
        return self._h

    @property
    def ncell(self):
        return lib().mpcd_cell_count(self._h)

    def set_fluid(self, pos, vel):
        pos, vel = _f64(pos), _f64(vel)
        self._ck(lib().mpcd_set_fluid(self._h, pos.shape[0], _dp(pos), _dp(vel)), "set_fluid")

    def fluid(self, out=None):
        """(pos, vel) as n x 3 float64 arrays; out=(pos, vel) fills given
        C-contiguous float64 arrays of that shape (e.g. pinned ones)."""
        n = lib().mpcd_fluid_count(self._h)
        if out is None:
            pos = np.zeros((n, 3))
            vel = np.zeros((n, 3))
        else:
            pos, vel = out
            for a in (pos, vel):
                if a.shape != (n, 3) or a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
                    raise ValueError(f"fluid: out arrays must be C-contiguous float64 of shape ({n}, 3)")
        self._ck(lib().mpcd_get_fluid(self._h, n, _dp(pos), _dp(vel)), "get_fluid")
        return pos, vel

    def pin(self, a):
        """Page-locks a C-contiguous numpy array for direct DMA copies; unpin
        it before it is freed."""
        if not a.flags["C_CONTIGUOUS"] or a.nbytes == 0:
            raise ValueError("pin: needs a non-empty C-contiguous array")
        self._ck(lib().mpcd_pin_host(self._h, a.ctypes.data, a.nbytes), "pin_host")
        return a

    def unpin(self, a):
        self._ck(lib().mpcd_unpin_host(self._h, a.ctypes.data), "unpin_host")

    @property
    def shift(self):
        a = np.zeros(3)
        self._ck(lib().mpcd_get_shift(self._h, _dp(a)), "get_shift")
        return a

    @shift.setter
    def shift(self, a):
        a = _f64(a)
        self._ck(lib().mpcd_set_shift(self._h, _dp(a)), "set_shift")

    @property
    def time(self):
        t = ctypes.c_double()
        self._ck(lib().mpcd_get_time(self._h, ctypes.byref(t)), "get_time")
        return t.value

    @time.setter
    def time(self, t):
        self._ck(lib().mpcd_set_time(self._h, float(t)), "set_time")

    def set_beads(self, pos, vel, moves=None):
        pos, vel = _f64(pos), _f64(vel)
        mv = None if moves is None else np.ascontiguousarray(moves, dtype=np.int32)
        self._ck(lib().mpcd_set_beads(self._h, pos.shape[0], _dp(pos), _dp(vel),
                                      None if mv is None else mv.ctypes.data_as(_IP)), "set_beads")

    def beads(self, n):
        pos = np.zeros((n, 3))
        vel = np.zeros((n, 3))
        self._ck(lib().mpcd_get_beads(self._h, n, _dp(pos), _dp(vel)), "get_beads")
        return pos, vel

    def prepare(self):
        self._ck(lib().mpcd_prepare(self._h), "prepare")

    def step(self, shift_next=None, gamma=None, axis=None, virt=None):
        if shift_next is None and gamma is None and axis is None and virt is None:
            self._ck(lib().mpcd_step(self._h, None), "step")
            return
        keep = [_f64(shift_next), _f64(gamma), _f64(axis), _f64(virt)]
        inj = MpcdInject(_dp(keep[0]), _dp(keep[1]), _dp(keep[2]), _dp(keep[3]))
        self._ck(lib().mpcd_step(self._h, ctypes.byref(inj)), "step")

    def run(self, nsteps):
        self._ck(lib().mpcd_run(self._h, int(nsteps)), "run")

    def sync(self):
        self._ck(lib().mpcd_sync(self._h), "sync")

    def observables(self):
        o = MpcdObs()
        self._ck(lib().mpcd_observables(self._h, ctypes.byref(o)), "observables")
        return dict(momentum=np.array(o.momentum[:]), n=o.n, mass=o.mass, kT=o.kT, fluid_T=o.fluid_T,
                    diss_energy=o.diss_energy, globalt=o.globalt, energy_fluid=o.energy_fluid)

    def observables_async(self):
        """Enqueues the observables of the current state; returns a ticket for
        observables_result (the newest OBS_RING tickets stay collectable)."""
        t = ctypes.c_longlong(0)
        self._ck(lib().mpcd_observables_async(self._h, ctypes.byref(t)), "observables_async")
        return t.value

    def observables_result(self, ticket):
        o = MpcdObs()
        self._ck(lib().mpcd_observables_result(self._h, ticket, ctypes.byref(o)), "observables_result")
        return dict(momentum=np.array(o.momentum[:]), n=o.n, mass=o.mass, kT=o.kT, fluid_T=o.fluid_T,
                    diss_energy=o.diss_energy, globalt=o.globalt, energy_fluid=o.energy_fluid)

    def reset_diss(self):
        self._ck(lib().mpcd_reset_diss(self._h), "reset_diss")

    def launch_count(self):
        return lib().mpcd_launch_count(self._h)

    def timed_run(self, nsteps, flush_l2=True):
        """Device time of each of `nsteps` free-running steps (ms)."""
        out = np.zeros(max(int(nsteps), 1))
        self._ck(lib().mpcd_timed_run(self._h, int(nsteps), int(flush_l2), _dp(out)), "timed_run")
        return out[: int(nsteps)]

    def set_profiling(self, on=True):
        self._ck(lib().mpcd_set_profiling(self._h, int(on)), "set_profiling")

    def kernel_time(self, kernel):
        """(total ms, launches) of one kernel class since profiling started."""
        ms = ctypes.c_double()
        n = ctypes.c_longlong()
        self._ck(lib().mpcd_kernel_time(self._h, int(kernel), ctypes.byref(ms), ctypes.byref(n)), "kernel_time")
        return ms.value, n.value

    def set_repelling(self, eps):
        """Contact forces between cilia (the reference's -DREPELLING=eps); 0 turns them off."""
        self._ck(lib().mpcd_set_repelling(self._h, float(eps)), "set_repelling")

    def snapshot(self):
        """The handle's whole state as bytes (mpcd_snapshot)."""
        n = ctypes.c_longlong()
        self._ck(lib().mpcd_snapshot_size(self._h, ctypes.byref(n)), "snapshot_size")
        buf = ctypes.create_string_buffer(n.value)
        self._ck(lib().mpcd_snapshot(self._h, buf, n.value), "snapshot")
        return buf.raw

    def restore(self, data):
        """Replace the handle's state by a snapshot (mpcd_restore)."""
        buf = ctypes.create_string_buffer(bytes(data), len(data))
        self._ck(lib().mpcd_restore(self._h, buf, len(data)), "restore")

    def set_rigid_spheres(self, spheres):
        """Rigid no-slip spheres: dicts with center, radius and optional velocity,
        omega, mass (> 0 free, <= 0 or absent held)."""
        arr = (MpcdRigidSphere * max(len(spheres), 1))()
        for k, sp in enumerate(spheres):
            arr[k].center[:] = [float(x) for x in sp["center"]]
            arr[k].velocity[:] = [float(x) for x in sp.get("velocity", (0.0, 0.0, 0.0))]
            arr[k].omega[:] = [float(x) for x in sp.get("omega", (0.0, 0.0, 0.0))]
            arr[k].radius = float(sp["radius"])
            arr[k].mass = float(sp.get("mass", 0.0))
        self._ck(lib().mpcd_set_rigid_spheres(self._h, len(spheres), arr), "set_rigid_spheres")

    def rigid_spheres(self):
        """(list of sphere dicts, mean force and torque [n, 6] since the last reset)."""
        n = lib().mpcd_rigid_sphere_count(self._h)
        arr = (MpcdRigidSphere * max(n, 1))()
        ft = np.zeros((max(n, 1), 6))
        self._ck(lib().mpcd_get_rigid_spheres(self._h, n, arr, _dp(ft)), "get_rigid_spheres")
        out = [dict(center=np.array(arr[k].center[:]), velocity=np.array(arr[k].velocity[:]),
                    omega=np.array(arr[k].omega[:]), radius=arr[k].radius, mass=arr[k].mass) for k in range(n)]
        return out, ft[:n]

    def reset_sphere_forces(self):
        self._ck(lib().mpcd_reset_rigid_sphere_forces(self._h), "reset_rigid_sphere_forces")

    def md_layout(self):
        """The MD kernels' layout: cluster or cooperative grid, threads per slot, tile, tiles, slots, springs."""
        a = (ctypes.c_int * 8)()
        self._ck(lib().mpcd_md_layout(self._h, a), "md_layout")
        keys = ("cluster", "lanes", "tile", "ntiles", "nslots", "nsprings", "hmax", "arith")
        return dict(zip(keys, list(a)))


def cfg_host_state(cfg, *, is_text=True, seed=1, create_fluid=True, read_files=False):
    """The initial state a sim.cfg describes, built on the host only (no GPU):
    dict(shift, fluid_pos, fluid_vel, bead_pos, bead_vel, nsprings)."""
    o = CiliaOptions(MPCD_FP64, 0, seed, 0.0, int(create_fluid), int(read_files), WALLS_NONE, 0.0, 5.0, 0, 0)
    text = cfg.encode() if isinstance(cfg, str) else cfg
    sizes = (ctypes.c_long * 3)()

    def call(*arrays):
        rc = lib().cilia_cfg_host_state(text, int(is_text), ctypes.byref(o), sizes, *arrays)
        if rc:
            msg = lib().cilia_sim_last_error(None)
            raise MpcdError(f"cilia_cfg_host_state failed ({rc}): {msg.decode() if msg else ''}")

    call(None, None, None, None, None)
    nf, nb = sizes[0], sizes[1]
    shift = np.zeros(3)
    fp, fv, bp, bv = np.zeros((nf, 3)), np.zeros((nf, 3)), np.zeros((nb, 3)), np.zeros((nb, 3))
    call(_dp(shift), _dp(fp), _dp(fv), _dp(bp), _dp(bv))
    return dict(shift=shift, fluid_pos=fp, fluid_vel=fv, bead_pos=bp, bead_vel=bv, nsprings=sizes[2])


class Sim:
    """The reference's Simulation on the GPU (cilia_sim), from cfg text or a path."""

    def __init__(self, cfg, *, is_text=True, precision=MPCD_FP64, seed=1, ststep=0.0, create_fluid=True,
                 read_files=False, walls=WALLS_NONE, gravity=0.0, bead_mass=5.0, device=0, sort_interval=0,
                 md_arith=MD_AUTO):
        o = CiliaOptions(precision, device, seed, ststep, int(create_fluid), int(read_files), walls, gravity,
                         bead_mass, sort_interval, int(md_arith) + 1)
        h = ctypes.c_void_p()
        rc = lib().cilia_sim_create(cfg.encode() if isinstance(cfg, str) else cfg, int(is_text),
                                    ctypes.byref(o), ctypes.byref(h))
        if rc:
            msg = lib().cilia_sim_last_error(None)
            raise MpcdError(f"cilia_sim_create failed ({rc}): {msg.decode() if msg else ''}")
        self._h = h
        self.engine = Engine(None, _handle=lib().cilia_sim_engine(h), _owner=self)

    def close(self):
        if getattr(self, "_h", None):
            lib().cilia_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _ck(self, rc, what):
        if rc:
            msg = lib().cilia_sim_last_error(self._h)
            raise MpcdError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")

    def num_objects(self):
        return lib().cilia_sim_num_objects(self._h)

    def object_info(self, i):
        info = (ctypes.c_int * 5)()
        name = ctypes.create_string_buffer(256)
        self._ck(lib().cilia_sim_object_info(self._h, i, info, name, 256), "object_info")
        return dict(rods=info[0], len=info[1], startidx=info[2], offset=info[3],
                    type=["Sphere", "Cilia", "ConstantBeatCilia", "Clami"][info[4]], name=name.value.decode())

    @property
    def nbeads(self):
        return lib().cilia_sim_bead_count(self._h)

    def beads(self):
        return self.engine.beads(self.nbeads)

    def next_tstep(self, shift_next=None, gamma=None, axis=None, virt=None):
        if shift_next is None and gamma is None and axis is None and virt is None:
            self._ck(lib().cilia_sim_next_tstep(self._h, None), "next_tstep")
            return
        keep = [_f64(shift_next), _f64(gamma), _f64(axis), _f64(virt)]
        inj = MpcdInject(_dp(keep[0]), _dp(keep[1]), _dp(keep[2]), _dp(keep[3]))
        self._ck(lib().cilia_sim_next_tstep(self._h, ctypes.byref(inj)), "next_tstep")

    def run(self):
        self._ck(lib().cilia_sim_run(self._h), "run")

    def save(self):
        self._ck(lib().cilia_sim_save(self._h), "save")

    def writedata(self, objects=True, debug=False):
        """The writes of a measure interval (cilia_sim_writedata) in the working directory."""
        self._ck(lib().cilia_sim_writedata(self._h, int(objects) | (2 if debug else 0)), "writedata")

    def write_cfg(self, path):
        self._ck(lib().cilia_sim_write_cfg(self._h, path.encode()), "write_cfg")


class Batch:
    """Many independent split-precision boxes advanced together (mpcd_batch)."""

    def __init__(self, *, max_replicas, max_particles, max_cells, max_slots=0, max_springs=0, max_halo=0,
                 max_cilia=0, max_bonds=0, md_lanes=0, md_tile=0, sort_interval=0, sorts_per_graph=0, device=0):
        p = MpcdBatchParams(device, max_replicas, max_particles, max_cells, max_slots, max_springs, max_halo,
                            max_cilia, max_bonds, md_lanes, md_tile, sort_interval, sorts_per_graph)
        h = ctypes.c_void_p()
        rc = lib().mpcd_batch_create(ctypes.byref(p), ctypes.byref(h))
        if rc:
            raise MpcdError(f"mpcd_batch_create failed with code {rc}")
        self._h = h

    @classmethod
    def for_specs(cls, specs, extra_replicas=2, **kw):
        """A batch with room for replicas of the given shapes (dicts with L,
        n_cilia, rodlength; a Clami sphere of 643 beads each when n_cilia is
        given, no beads when `beads` is False)."""
        nf = sum(10 * s["L"] ** 3 for s in specs)
        nc = sum(s["L"] ** 3 for s in specs)
        nb = sum((643 + 3 * s["n_cilia"] * s["rodlength"]) if s.get("beads", True) else 0 for s in specs)
        k = len(specs)
        args = dict(max_replicas=k + extra_replicas, max_particles=nf + 8192 * k, max_cells=nc + 2048 * k,
                    max_slots=2 * nb + 1024 * k, max_springs=14 * nb + 1, max_halo=6 * nb + 4096,
                    max_cilia=sum(s["n_cilia"] for s in specs) + 1,
                    max_bonds=sum(s["n_cilia"] * s["rodlength"] for s in specs) + 1)
        args.update(kw)
        return cls(**args)

    def close(self):
        if getattr(self, "_h", None):
            lib().mpcd_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _ck(self, rc, what):
        if rc:
            msg = lib().mpcd_batch_last_error(self._h)
            raise MpcdError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")

    def add(self, L, *, tstep=0.1, ststep=0.002, bead_mass=5.0, seed=1, gravity=0.0, omega=0.0):
        if isinstance(L, int):
            L = (L, L, L)
        p = MpcdParams()
        p.sizes[:] = [int(x) for x in L]
        p.tstep, p.ststep, p.precision, p.walls = tstep, ststep, MPCD_FP32, WALLS_NONE
        p.gravity, p.omega, p.bead_mass, p.seed = gravity, omega, bead_mass, seed
        r = ctypes.c_int()
        self._ck(lib().mpcd_batch_add(self._h, ctypes.byref(p), ctypes.byref(r)), "batch_add")
        return r.value

    def add_engine(self, engine):
        r = ctypes.c_int()
        self._ck(lib().mpcd_batch_add_engine(self._h, engine.handle, ctypes.byref(r)), "batch_add_engine")
        return r.value

    def add_cfg(self, cfg, *, is_text=True, seed=1, ststep=0.0, bead_mass=5.0, create_fluid=True):
        """A replica built on the host from a sim.cfg (not yet admitted)."""
        o = CiliaOptions(MPCD_FP32, 0, seed, ststep, int(create_fluid), 0, WALLS_NONE, 0.0, bead_mass, 0, 0)
        r = ctypes.c_int()
        rc = lib().cilia_batch_add_cfg(self._h, cfg.encode() if isinstance(cfg, str) else cfg, int(is_text),
                                       ctypes.byref(o), ctypes.byref(r))
        if rc:
            m1 = lib().cilia_sim_last_error(None)
            m2 = lib().mpcd_batch_last_error(self._h)
            raise MpcdError(f"cilia_batch_add_cfg failed ({rc}): {(m1 or b'').decode()} {(m2 or b'').decode()}")
        return r.value

    def set_fluid(self, r, pos, vel):
        pos, vel = _f64(pos), _f64(vel)
        self._ck(lib().mpcd_batch_set_fluid(self._h, r, pos.shape[0], _dp(pos), _dp(vel)), "batch_set_fluid")

    def set_shift(self, r, a):
        a = _f64(a)
        self._ck(lib().mpcd_batch_set_shift(self._h, r, _dp(a)), "batch_set_shift")

    def shift(self, r):
        a = np.zeros(3)
        self._ck(lib().mpcd_batch_get_shift(self._h, r, _dp(a)), "batch_get_shift")
        return a

    def footprint(self, r):
        v = ctypes.c_longlong()
        self._ck(lib().mpcd_batch_footprint(self._h, r, ctypes.byref(v)), "batch_footprint")
        return v.value

    def admit(self, r):
        self._ck(lib().mpcd_batch_admit(self._h, r), "batch_admit")

    def try_admit(self, r):
        return lib().mpcd_batch_admit(self._h, r) == 0

    def set_steps(self, r, n):
        self._ck(lib().mpcd_batch_set_steps(self._h, r, int(n)), "batch_set_steps")

    def run(self, nsteps):
        self._ck(lib().mpcd_batch_run(self._h, int(nsteps)), "batch_run")

    def step_inject(self, r, shift_next=None, gamma=None, axis=None):
        """One step in which replica r takes injected randomness (mpcd_batch_step_inject)."""
        keep = [_f64(shift_next), _f64(gamma), _f64(axis)]
        inj = MpcdInject(_dp(keep[0]), _dp(keep[1]), _dp(keep[2]), None)
        self._ck(lib().mpcd_batch_step_inject(self._h, r, ctypes.byref(inj)), "step_inject")

    def timed_run(self, nsteps):
        ms = ctypes.c_double()
        self._ck(lib().mpcd_batch_timed_run(self._h, int(nsteps), ctypes.byref(ms)), "batch_timed_run")
        return ms.value

    def sync(self):
        self._ck(lib().mpcd_batch_sync(self._h), "batch_sync")

    def status(self, r):
        d, left, err = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_uint()
        t = ctypes.c_double()
        self._ck(lib().mpcd_batch_status(self._h, r, ctypes.byref(d), ctypes.byref(left), ctypes.byref(t),
                                         ctypes.byref(err)), "batch_status")
        return dict(steps=d.value, steps_left=left.value, globalt=t.value, err=err.value)

    def fluid(self, r, n):
        pos = np.zeros((n, 3))
        vel = np.zeros((n, 3))
        self._ck(lib().mpcd_batch_get_fluid(self._h, r, n, _dp(pos), _dp(vel)), "batch_get_fluid")
        return pos, vel

    def beads(self, r, n):
        pos = np.zeros((n, 3))
        vel = np.zeros((n, 3))
        self._ck(lib().mpcd_batch_get_beads(self._h, r, n, _dp(pos), _dp(vel)), "batch_get_beads")
        return pos, vel

    def observables(self, r):
        o = MpcdObs()
        self._ck(lib().mpcd_batch_observables(self._h, r, ctypes.byref(o)), "batch_observables")
        return dict(momentum=np.array(o.momentum[:]), n=o.n, mass=o.mass, kT=o.kT, fluid_T=o.fluid_T,
                    diss_energy=o.diss_energy, globalt=o.globalt, energy_fluid=o.energy_fluid)

    def remove(self, r):
        self._ck(lib().mpcd_batch_remove(self._h, r), "batch_remove")

    @property
    def resident(self):
        return lib().mpcd_batch_resident(self._h)

    def autotune(self, trial_steps=50):
        t = MpcdBatchTuning()
        self._ck(lib().mpcd_batch_autotune(self._h, int(trial_steps), ctypes.byref(t)), "batch_autotune")
        lanes, tile = self.md_layout()
        return dict(fluid_threads=t.fluid_threads, fluid_blocks=t.fluid_blocks, cell_threads=t.cell_threads,
                    cell_blocks=t.cell_blocks, sort_interval=t.sort_interval, md_lanes=lanes, md_tile=tile)

    def tuning(self):
        t = MpcdBatchTuning()
        self._ck(lib().mpcd_batch_get_tuning(self._h, ctypes.byref(t)), "batch_get_tuning")
        return dict(fluid_threads=t.fluid_threads, fluid_blocks=t.fluid_blocks, cell_threads=t.cell_threads,
                    cell_blocks=t.cell_blocks, sort_interval=t.sort_interval)

    def set_tuning(self, **kw):
        cur = self.tuning()
        cur.update(kw)
        t = MpcdBatchTuning(cur["fluid_threads"], cur["fluid_blocks"], cur["cell_threads"], cur["cell_blocks"],
                            cur["sort_interval"])
        self._ck(lib().mpcd_batch_set_tuning(self._h, ctypes.byref(t)), "batch_set_tuning")

    def launch_count(self):
        return lib().mpcd_batch_launch_count(self._h)

    def set_md_layout(self, lanes, tile):
        self._ck(lib().mpcd_batch_set_md_layout(self._h, int(lanes), int(tile)), "batch_set_md_layout")

    def md_layout(self):
        a, t = ctypes.c_int(), ctypes.c_int()
        self._ck(lib().mpcd_batch_get_md_layout(self._h, ctypes.byref(a), ctypes.byref(t)), "batch_get_md_layout")
        return a.value, t.value

    def stage_times(self, nsteps=10):
        """Device ms per step of (cell maps, fluid pass, MD, sorts), stages serialised."""
        out = np.zeros(4)
        self._ck(lib().mpcd_batch_stage_times(self._h, int(nsteps), _dp(out)), "batch_stage_times")
        return dict(cell=out[0], fluid=out[1], md=out[2], sort=out[3])


def _info_dict(i):
    o = i.obs
    return dict(id=i.id, state=i.state, steps=i.steps, t_submit=i.t_submit, t_admit=i.t_admit, t_done=i.t_done,
                nfluid=i.nfluid, nbeads=i.nbeads, footprint=i.footprint, err=i.err_bits, preemptions=i.preemptions,
                obs=dict(momentum=np.array(o.momentum[:]), n=o.n, mass=o.mass, kT=o.kT, fluid_T=o.fluid_T,
                         diss_energy=o.diss_energy, globalt=o.globalt, energy_fluid=o.energy_fluid))


class Server:
    """Continuous batching of swimmer runs (mpcd_server)."""

    def __init__(self, *, budget_bytes=0, chunk_steps=0, keep_fluid=False, lookahead=0, prep_threads=0,
                 preempt_wait_s=0.0, **batch):
        b = dict(device=0, max_replicas=16, max_particles=0, max_cells=0, max_slots=0, max_springs=0, max_halo=0,
                 max_cilia=0, max_bonds=0, md_lanes=0, md_tile=0, sort_interval=0, sorts_per_graph=0)
        b.update(batch)
        p = MpcdServerParams(MpcdBatchParams(b["device"], b["max_replicas"], b["max_particles"], b["max_cells"],
                                             b["max_slots"], b["max_springs"], b["max_halo"], b["max_cilia"],
                                             b["max_bonds"], b["md_lanes"], b["md_tile"], b["sort_interval"],
                                             b["sorts_per_graph"]),
                             int(budget_bytes), int(chunk_steps), int(bool(keep_fluid)), int(lookahead),
                             int(prep_threads), float(preempt_wait_s))
        h = ctypes.c_void_p()
        rc = lib().mpcd_server_create(ctypes.byref(p), ctypes.byref(h))
        if rc:
            raise MpcdError(f"mpcd_server_create failed with code {rc}")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().mpcd_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def submit(self, cfg, nsteps, seed=1):
        i = ctypes.c_longlong()
        rc = lib().mpcd_server_submit(self._h, cfg.encode() if isinstance(cfg, str) else cfg, int(nsteps), int(seed),
                                      ctypes.byref(i))
        if rc:
            raise MpcdError(f"submit failed ({rc})")
        return i.value

    def info(self, rid):
        i = MpcdRequestInfo()
        if lib().mpcd_server_info(self._h, int(rid), ctypes.byref(i)):
            raise MpcdError("unknown request")
        return _info_dict(i)

    def wait(self, rid, timeout=600.0):
        """Info of the finished request; raises if it failed or timed out."""
        i = MpcdRequestInfo()
        rc = lib().mpcd_server_wait(self._h, int(rid), float(timeout), ctypes.byref(i))
        if rc:
            msg = lib().mpcd_server_last_error(self._h)
            raise MpcdError(f"request {rid}: wait failed ({rc}): {self.error(rid) or (msg.decode() if msg else '')}")
        return _info_dict(i)

    def drain(self, timeout=600.0):
        if lib().mpcd_server_drain(self._h, float(timeout)):
            raise MpcdError("drain timed out")

    def result_beads(self, rid, nb):
        pos, vel = np.zeros((nb, 3)), np.zeros((nb, 3))
        if lib().mpcd_server_result_beads(self._h, int(rid), int(nb), _dp(pos), _dp(vel)):
            raise MpcdError("no bead result")
        return pos, vel

    def result_fluid(self, rid, n):
        pos, vel = np.zeros((n, 3)), np.zeros((n, 3))
        if lib().mpcd_server_result_fluid(self._h, int(rid), int(n), _dp(pos), _dp(vel)):
            raise MpcdError("no fluid result")
        return pos, vel

    def preempt(self, rid):
        """Pre-empt a resident request at the end of the round (mpcd_server_preempt); False if not resident."""
        return lib().mpcd_server_preempt(self._h, int(rid)) == 0

    def error(self, rid):
        m = lib().mpcd_server_request_error(self._h, int(rid))
        return m.decode() if m else ""

    def stats(self):
        st = MpcdServerStats()
        lib().mpcd_server_get_stats(self._h, ctypes.byref(st))
        return {k: getattr(st, k) for k, _ in MpcdServerStats._fields_}
