"""ctypes wrapper around the C oracle (oracle/mpcd_oracle.c).

Test infrastructure: imported only by tests/, the smoke check and bench.py's
CPU-baseline leg, as the checker.  The library is built by ``make -C oracle``
into ``oracle/_build/liboracle.so``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_D = ctypes.c_double
_I = ctypes.c_int
_L = ctypes.c_long
_P = ctypes.c_void_p
_DP = ctypes.POINTER(ctypes.c_double)


def build() -> str:
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.orc_create.restype = _P
        L.orc_create.argtypes = [_I, _I, _I, _D, _D, ctypes.c_uint]
        L.orc_destroy.argtypes = [_P]
        L.orc_mt_next.restype = ctypes.c_uint
        L.orc_mt_next.argtypes = [_P]
        L.orc_rgamma.restype = _D
        L.orc_rgamma.argtypes = [_P, _I]
        for name in ("orc_init_shift", "orc_fluid_create", "orc_init_bins", "orc_reset_diss"):
            getattr(L, name).argtypes = [_P]
        L.orc_set_shift.argtypes = [_P, _DP]
        L.orc_get_shift.argtypes = [_P, _DP]
        L.orc_set_globalt.argtypes = [_P, _D]
        L.orc_get_globalt.restype = _D
        L.orc_get_globalt.argtypes = [_P]
        L.orc_fluid_set.restype = _I
        L.orc_fluid_set.argtypes = [_P, _L, _DP, _DP]
        L.orc_fluid_count.restype = _L
        L.orc_fluid_count.argtypes = [_P]
        L.orc_fluid_get.argtypes = [_P, _DP, _DP]
        L.orc_add_sphere.restype = _I
        L.orc_add_sphere.argtypes = [_P, _D, _D, _D, _D, _D, _I]
        L.orc_add_cilia.restype = _I
        L.orc_add_cilia.argtypes = [_P, _I, _I, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _I, _I, _D, _D, _D]
        L.orc_add_clami.restype = _I
        L.orc_add_clami.argtypes = [_P, _D, _D, _D, _D, _D, _I, ctypes.POINTER(_I), _DP, _DP, _DP,
                                    _I, _I, _D, _D, _D, _D, _D, _D, _D, _D, _D]
        L.orc_num_objects.restype = _I
        L.orc_num_objects.argtypes = [_P]
        L.orc_object_info.argtypes = [_P, _I, ctypes.POINTER(_I)]
        L.orc_bead_count.restype = _L
        L.orc_bead_count.argtypes = [_P]
        L.orc_beads_get.argtypes = [_P, _DP, _DP]
        L.orc_beads_set.restype = _I
        L.orc_beads_set.argtypes = [_P, _DP, _DP]
        L.orc_cilium_state.restype = _I
        L.orc_cilium_state.argtypes = [_P, _I, _DP]
        L.orc_sphere_headbond.restype = _D
        L.orc_sphere_headbond.argtypes = [_P, _I]
        L.orc_clami_springs.restype = _I
        L.orc_clami_springs.argtypes = [_P, _I, _DP, _I]
        L.orc_step.restype = _I
        L.orc_step.argtypes = [_P, _DP, _DP, _DP, _DP, _DP, _DP]
        L.orc_step_walls.restype = _I
        L.orc_step_walls.argtypes = [_P, _DP, _DP, _DP, _DP, _DP, _DP, _DP, _DP]
        L.orc_set_walls.argtypes = [_P, _I]
        L.orc_set_gravity.argtypes = [_P, _D, _D]
        L.orc_set_repelling.argtypes = [_P, _D]
        L.orc_contacts.restype = _L
        L.orc_contacts.argtypes = [_P]
        L.orc_diss_energy.restype = _D
        L.orc_diss_energy.argtypes = [_P]
        L.orc_set_threads.argtypes = [_P, _I]
        L.orc_observables.argtypes = [_P, _DP]
        _lib = L
    return _lib


def _ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(_DP)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class OracleSim:
    """One reference-equivalent simulation (MPCD + MD objects) on the CPU."""

    def __init__(self, L, tstep=0.1, ststep=0.001, seed=1):
        if isinstance(L, int):
            L = (L, L, L)
        self.L = tuple(int(x) for x in L)
        self.ncell = self.L[0] * self.L[1] * self.L[2]
        self._h = lib().orc_create(self.L[0], self.L[1], self.L[2], float(tstep), float(ststep), int(seed))

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    # --- generator
    def mt_next(self):
        return lib().orc_mt_next(self._h)

    def rgamma(self, nc):
        return lib().orc_rgamma(self._h, int(nc))

    # --- shift / time
    def init_shift(self):
        lib().orc_init_shift(self._h)

    @property
    def shift(self):
        a = np.zeros(3)
        lib().orc_get_shift(self._h, _ptr(a))
        return a

    @shift.setter
    def shift(self, a):
        a = _f64(a)
        lib().orc_set_shift(self._h, _ptr(a))

    @property
    def globalt(self):
        return lib().orc_get_globalt(self._h)

    @globalt.setter
    def globalt(self, t):
        lib().orc_set_globalt(self._h, float(t))

    # --- fluid
    def fluid_create(self):
        lib().orc_fluid_create(self._h)

    def fluid_set(self, pos, vel):
        pos, vel = _f64(pos), _f64(vel)
        lib().orc_fluid_set(self._h, pos.shape[0], _ptr(pos), _ptr(vel))

    def fluid(self):
        n = lib().orc_fluid_count(self._h)
        pos = np.zeros((n, 3))
        vel = np.zeros((n, 3))
        lib().orc_fluid_get(self._h, _ptr(pos), _ptr(vel))
        return pos, vel

    # --- MD objects
    def add_sphere(self, radius, k, position, npart=643):
        return lib().orc_add_sphere(self._h, radius, k, *[float(x) for x in position], int(npart))

    def add_cilia(self, *, kind, rodlength, beatstrength, bending, min_bend, max_bend, m_speed,
                  springconstant, position, thetaX, thetaY, thetaZ, startidx=0, num_anker=2,
                  power_stroke_duration=0.0, recovery_stroke_duration=0.0, start_delay=0.0):
        return lib().orc_add_cilia(self._h, int(kind), int(rodlength), beatstrength, bending, min_bend,
                                   max_bend, m_speed, springconstant, *[float(x) for x in position],
                                   thetaX, thetaY, thetaZ, int(startidx), int(num_anker),
                                   power_stroke_duration, recovery_stroke_duration, start_delay)

    def add_clami(self, *, radius, springconstant, position, num_equators, y_thetas, theta_offset,
                  start_delays=None, cilia):
        ne = (ctypes.c_int * len(num_equators))(*[int(x) for x in num_equators])
        yt = _f64(y_thetas)
        to = _f64(theta_offset)
        sd = None if start_delays is None else _f64(start_delays)
        c = cilia
        kind = 1 if c.get("type", "ConstantBeatCilia") == "ConstantBeatCilia" else 0
        return lib().orc_add_clami(
            self._h, radius, springconstant, *[float(x) for x in position], len(num_equators), ne,
            _ptr(yt), _ptr(to), _ptr(sd), kind, int(c["rodlength"]), c["beatstrength"], c["bending"],
            c["min_bend"], c["max_bend"], c["m_speed"], c["springconstant"], c.get("thetaZ", 0.0),
            c.get("power_stroke_duration", 0.0), c.get("recovery_stroke_duration", 0.0))

    def num_objects(self):
        return lib().orc_num_objects(self._h)

    def object_info(self, i):
        info = (ctypes.c_int * 5)()
        lib().orc_object_info(self._h, i, info)
        return dict(kind=info[0], rods=info[1], len=info[2], startidx=info[3], offset=info[4])

    def bead_count(self):
        return lib().orc_bead_count(self._h)

    def beads(self):
        n = self.bead_count()
        pos = np.zeros((n, 3))
        vel = np.zeros((n, 3))
        if n:
            lib().orc_beads_get(self._h, _ptr(pos), _ptr(vel))
        return pos, vel

    def beads_set(self, pos=None, vel=None):
        lib().orc_beads_set(self._h, _ptr(None if pos is None else _f64(pos)),
                            _ptr(None if vel is None else _f64(vel)))

    def cilium_state(self, obj):
        info = self.object_info(obj)
        out = np.zeros(2 * info["len"] + 2)
        lib().orc_cilium_state(self._h, obj, _ptr(out))
        return out

    def sphere_headbond(self, obj):
        return lib().orc_sphere_headbond(self._h, obj)

    def clami_springs(self, obj):
        n = lib().orc_clami_springs(self._h, obj, None, 0)
        out = np.zeros((max(n, 1), 5))
        lib().orc_clami_springs(self._h, obj, _ptr(out), n)
        return out[:n]

    def init_bins(self):
        lib().orc_init_bins(self._h)

    # --- stepping
    def set_walls(self, walls):
        """0 periodic, 1 no-slip, 2 slip walls at z = 0 and z = Lz - 1."""
        lib().orc_set_walls(self._h, int(walls))

    def set_gravity(self, g, omega=0.0):
        lib().orc_set_gravity(self._h, float(g), float(omega))

    def set_repelling(self, eps):
        """Contact forces between cilia (the reference's -DREPELLING=eps)."""
        lib().orc_set_repelling(self._h, float(eps))

    def contacts(self):
        return lib().orc_contacts(self._h)

    def step(self, shift_next=None, gamma=None, axis=None, record=False, virt=None):
        """One MPC step; with record=True returns (shift, gamma, axis, virt) as drawn."""
        rs = rg = ra = rv = None
        if record:
            rs = np.zeros(3)
            rg = np.full(self.ncell, -2.0)
            ra = np.zeros((self.ncell, 3))
            rv = np.zeros((self.ncell, 3))
        sn = None if shift_next is None else _f64(shift_next)
        g = None if gamma is None else _f64(gamma)
        ax = None if axis is None else _f64(axis)
        vv = None if virt is None else _f64(virt)
        err = lib().orc_step_walls(self._h, _ptr(sn), _ptr(g), _ptr(ax), _ptr(vv), _ptr(rs), _ptr(rg), _ptr(ra),
                                   _ptr(rv))
        if err:
            raise RuntimeError("oracle step: injected gamma missing for a thermostatted cell")
        if record:
            return rs, rg, ra, rv
        return None

    def diss_energy(self):
        return lib().orc_diss_energy(self._h)

    def set_threads(self, t):
        lib().orc_set_threads(self._h, int(t))

    def observables(self):
        out = np.zeros(6)
        lib().orc_observables(self._h, _ptr(out))
        return dict(momentum=out[0:3].copy(), n=int(out[3]), mass=out[4], kT=out[5])


def build_from_cfg(cfg: dict, seed: int, ststep: float | None = None, create_fluid: bool = True) -> OracleSim:
    """Construct the reference's Simulation(root) from a parsed sim.cfg.

    Order of construction and random draws follows src/simulation.cpp:19-35:
    MPCD (initial grid shift), md_objects in list order (no draws), fluid
    creation, then MDObject::init binning.
    """
    if ststep is None:
        ststep = float(cfg.get("ststep", 0.001))
    L = (int(cfg["sizex"]), int(cfg["sizey"]), int(cfg["sizez"]))
    s = OracleSim(L, tstep=float(cfg["tstep"]), ststep=ststep, seed=seed)
    s.globalt = float(cfg["globalt"])
    s.init_shift()
    for o in cfg["md_objects"]:
        t = o["type"]
        if t == "Sphere":
            s.add_sphere(o["radius"], o["springconstant"], o["position"], o["npart"])
        elif t in ("Cilia", "ConstantBeatCilia"):
            s.add_cilia(kind=1 if t == "ConstantBeatCilia" else 0, rodlength=o["rodlength"],
                        beatstrength=o["beatstrength"], bending=o["bending"], min_bend=o["min_bend"],
                        max_bend=o["max_bend"], m_speed=o["m_speed"], springconstant=o["springconstant"],
                        position=o["position"], thetaX=o["thetaX"], thetaY=o["thetaY"], thetaZ=o["thetaZ"],
                        power_stroke_duration=o.get("power_stroke_duration", 0.0),
                        recovery_stroke_duration=o.get("recovery_stroke_duration", 0.0),
                        start_delay=o.get("start_delay", 0.0))
        elif t == "Clami":
            s.add_clami(radius=o["radius"], springconstant=o.get("springconstant", 20000.0),
                        position=o["position"], num_equators=o["num_equators"], y_thetas=o["y_thetas"],
                        theta_offset=o["theta_offset"], start_delays=o.get("start_delays"),
                        cilia=o["cilia"])
        else:
            raise ValueError(f"unknown md object type {t}")
    if create_fluid:
        s.fluid_create()
    s.init_bins()
    return s
