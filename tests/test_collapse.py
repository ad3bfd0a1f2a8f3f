"""The oracle's collapse physics (collapse.f90) against a second, numpy
restatement of the fits of collapse.f90:177-381 (CPU).  The collapse module
has no output file in the reference's examples; this cross-check of the two
restatements guards the density and Av the fixture of tests/golden/
collapse_modes.npz carries: the parcel density at t = 0 for every mode,
density at every row for the modes whose parcel stays at rout (filament,
ambipolar: the radius update's dt = targetTime - currentTime is zero), and
Av = baseAv + N/1.6e21 with N the trapezoid column of the profile."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

FIX = os.path.join(GOLDEN, "collapse_modes.npz")
SP = lambda x: float(np.float32(x))  # noqa: E731  (default-REAL literal)
MH, AU, PC, SPY = 1.67262164e-24, 2.063e5, 3.086e18, 3.16e7
PI = SP(3.141592654)
TMAX = {1: 1.175e6, 2: 1.855e5, 3: 0.0, 4: 0.0}
UNITT = (2 * PI * 6.67e-8 * 2.2e4 * MH) ** (-0.5) / SPY
UNITR = np.sqrt(1.38e-16 * 10 / 2 / MH) * (2 * PI * 6.67e-8 * 2.2e4 * MH) ** (-0.5) / PC


def fits(mode, t):
    """(rho0, r0, a) of collapse.f90:199-261."""
    tm = TMAX[mode]
    if mode == 1:
        l0 = SP(61.8) * (tm - t) ** SP(-0.01) - SP(49.4)
        l1 = -SP(28.5) * (tm - t) ** SP(-0.01) + SP(28.93)
        a = 2.4
    elif mode == 2:
        l0 = SP(68.4) * (tm - t) ** SP(-0.01) - SP(55.7)
        l1 = -SP(39.0) * (tm - t) ** SP(-0.01) + SP(38.7)
        a = SP(1.9) + 0.5 * np.exp(-t / 1e5)
    elif mode == 3:
        x = SP(5.47) - t / UNITT
        l0 = SP(3.54) * x ** SP(-0.15) - SP(2.73)
        l1 = -SP(1.34) * x ** SP(-0.15) + SP(1.47)
        a = 2.0 - 0.5 * (t / UNITT / SP(5.47)) ** 9
    else:
        x = SP(16.138) - 1e-6 * t
        l0 = None if t <= 6.0 else SP(5.3) * x ** SP(-0.1) - 1.0
        l1 = -SP(2.57) * x ** SP(-0.1) + SP(1.85)
        a = SP(2.4) - SP(0.2) * (1e-6 * t / SP(16.138)) ** 40
    rho0 = 2.0e3 + 1.7e3 * (t / 6.0 - 1.0) if l0 is None else 10.0 ** l0
    return rho0, 10.0 ** l1, a


def rho(mode, r, rho0, r0, a):
    r = np.asarray(r, dtype=np.float64)
    if mode in (1, 2):
        return rho0 / (1 + (r * AU / r0) ** a)
    if mode == 3:
        return 2.2e4 * rho0 / (1 + (r / UNITR / r0) ** 2) ** a
    return rho0 / (1 + (r / 0.75 / r0) ** a)


def coldens(mode, t, rin=0.0, rout=SP(0.05)):
    rho0, r0, a = fits(mode, t)
    x = rin + np.arange(10001) * ((rout - rin) / 10000)
    f = rho(mode, x, rho0, r0, a)
    return float(np.sum(0.5 * (f[1:] + f[:-1]) * ((rout - rin) / 10000) * PC))


@pytest.fixture(scope="module")
def fx():
    if not os.path.exists(FIX):
        pytest.fail(f"fixture missing: {FIX}")
    return np.load(FIX)


def test_initial_density_of_every_mode(fx):
    for k, mode in enumerate(fx["modes"]):
        rho0, r0, a = fits(int(mode), 0.0)
        np.testing.assert_allclose(fx["density"][k, 0], rho(int(mode), 0.0, rho0, r0, a), rtol=1e-12)


def test_density_and_av_of_the_fixed_parcel_modes(fx):
    """Filament and ambipolar: density(t) = rho(rout, fits(t)) and
    Av(t) = baseAv + N(t)/1.6e21 on every row after the first."""
    for k, mode in enumerate(fx["modes"]):
        n = int(fx["nrows"][k])
        for r in range(1, n, max(1, n // 12)):
            t = fx["tyears"][k, r]
            if int(mode) in (3, 4):
                rho0, r0, a = fits(int(mode), t)
                np.testing.assert_allclose(fx["density"][k, r], rho(int(mode), SP(0.05), rho0, r0, a), rtol=1e-10)
            np.testing.assert_allclose(fx["av"][k, r], SP(2.0) + coldens(int(mode), t) / 1.6e21, rtol=1e-10)


def test_bonnor_ebert_parcels_keep_their_mass(fx):
    """BE1.1 and BE4: the parcel's density on each row is the profile at
    the radius enclosing the initial mass (to the 1e4-step radius grid)."""
    for k, mode in enumerate(fx["modes"]):
        mode = int(mode)
        if mode not in (1, 2):
            continue
        rho0, r0, a = fits(mode, 0.0)
        rr = np.arange(1001) * (SP(0.05) / 1000)
        f = rho(mode, rr, rho0, r0, a)
        mass = float(np.sum(0.5 * (f[1:] + f[:-1]) * (SP(0.05) / 1000) * rr[1:] ** 2))
        n = int(fx["nrows"][k])
        for r in range(1, n, max(1, n // 8)):
            rho0, r0, a = fits(mode, fx["tyears"][k, r])
            grid = np.arange(1, 20001) * (SP(0.05) / 1.0e4)
            g = rho(mode, np.concatenate([[0.0], grid]), rho0, r0, a)
            m = np.cumsum(0.5 * (g[1:] + g[:-1]) * (SP(0.05) / 1.0e4) * grid ** 2)
            i = int(np.argmax(m >= mass))
            np.testing.assert_allclose(fx["density"][k, r], rho(mode, grid[i], rho0, r0, a), rtol=1e-3)


def test_collapse_and_hot_core_arguments_on_the_host():
    """model.collapse's argument rules (model.py:355-361) are checked before
    any device work, and the physics-module fields are not dictionary keys
    (dictionaryParser rejects unknown keys)."""
    from uclchem_gb300 import model
    from uclchem_gb300.params import ParameterError, make_params
    with pytest.raises(ValueError):
        model.collapse("BE5", None, {})
    with pytest.raises(ValueError):
        model.collapse("BE4", "physics.dat", {})
    for key in ("collapse", "hotcore", "maxTemperature"):
        with pytest.raises(ParameterError):
            make_params({key: 1})
    p = make_params({})
    assert p["collapse"] == 0 and p["hotcore"] == 0 and p["maxTemperature"] == 0.0
