"""Statistical parity of free-running (counter-based generator) GPU runs with
the C oracle (MT19937, the reference's generator): the two use different
random numbers, so they are compared through observables.

  - temperature kT after equilibration: within 0.01 of 1 on both;
  - velocity autocorrelation C(k) = <v(t0) . v(t0 + k h)> / <v(t0)^2> of the
    fluid for k = 1..8 MPC steps, averaged over 12 time origins: GPU and
    oracle within 0.006 of each other (the standard error of each is about
    0.001 here), for the float64 path and the float32 split path.  For SRD
    with a 130 degree rotation about a random axis and 10 particles per cell
    C(1) is about (1 - 1/10)(cos a + (1 - cos a)/3) + 1/10 = 0.015.
"""
import numpy as np
import pytest

import cilia_gpu as cg
from oracle import OracleSim

pytestmark = pytest.mark.gpu

L = (12, 12, 12)
LAGS = 8
ORIGINS = 12


def vacf(step, fluid):
    """C(k) for k = 0..LAGS, averaged over ORIGINS origins LAGS + 2 steps apart."""
    acc = np.zeros(LAGS + 1)
    for _ in range(ORIGINS):
        v0 = fluid()
        norm = np.mean(np.sum(v0 * v0, axis=1))
        for k in range(LAGS + 1):
            if k:
                step()
            acc[k] += np.mean(np.sum(v0 * fluid(), axis=1)) / norm
        step()
        step()
    return acc / ORIGINS


def oracle_run():
    o = OracleSim(L, tstep=0.1, ststep=0.002, seed=31)
    o.init_shift()
    o.fluid_create()
    o.set_threads(8)
    o.init_bins()
    for _ in range(50):
        o.step()
    c = vacf(lambda: o.step(), lambda: o.fluid()[1])
    return c, o.observables()["kT"]


@pytest.fixture(scope="module")
def oracle_vacf():
    return oracle_run()


@pytest.mark.parametrize("precision", [cg.MPCD_FP64, cg.MPCD_FP32])
def test_temperature_and_vacf_match_oracle(precision, oracle_vacf):
    c_orc, kt_orc = oracle_vacf
    o = OracleSim(L, tstep=0.1, ststep=0.002, seed=32)
    o.init_shift()
    o.fluid_create()
    p0, v0 = o.fluid()
    e = cg.Engine(L, tstep=0.1, ststep=0.002, precision=precision, seed=77)
    e.set_fluid(p0, v0)
    e.run(50)
    c_gpu = vacf(lambda: e.step(), lambda: e.fluid()[1])
    kt_gpu = e.observables()["kT"]
    assert abs(kt_gpu - 1.0) < 0.01 and abs(kt_orc - 1.0) < 0.01
    assert c_gpu[0] == pytest.approx(1.0) and c_orc[0] == pytest.approx(1.0)
    assert np.abs(c_gpu - c_orc).max() < 0.006, (c_gpu, c_orc)
    assert abs(c_orc[1] - 0.0148) < 0.006 and np.abs(c_gpu[1:]).max() < 0.1
