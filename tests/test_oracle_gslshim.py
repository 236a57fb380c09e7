"""The project's GSL-subset shim (oracle/gslshim/gslshim.c) against independent numerics (scipy).
GSL itself is absent, so this is how the shim's Ei, natural cubic spline, QAG GK41 and
nmsimplex2 are checked."""
import ctypes as C

import numpy as np
import pytest

import _oracle as O

scipy_special = pytest.importorskip("scipy.special")
scipy_integrate = pytest.importorskip("scipy.integrate")
scipy_interp = pytest.importorskip("scipy.interpolate")


@pytest.fixture(scope="module")
def lib():
    lib = O.load_oracle()
    lib.gsl_sf_expint_Ei.restype = C.c_double
    lib.gsl_sf_expint_Ei.argtypes = [C.c_double]
    return lib


def test_ei_against_mpmath(lib):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 30
    xs = np.concatenate([np.linspace(1e-4, 3, 50), np.linspace(3, 40, 200), np.linspace(40.0001, 120, 100),
                         -np.linspace(0.01, 30, 50)])
    for x in xs:
        assert lib.gsl_sf_expint_Ei(x) == pytest.approx(float(mp.ei(x)), rel=5e-15, abs=1e-16)


def test_position_marginal_matches_closed_form(lib):
    D = 0.5 * 5.991
    for x in (3.0, 5.0, 20.0, 60.0, 99.9):
        want = np.log((scipy_special.expi(x) - scipy_special.expi(x - D)) / np.log(x / (x - D)))
        assert lib.orc_marginalise_over_position_shift(x) == pytest.approx(want, rel=1e-13)
    assert lib.orc_marginalise_over_position_shift(2.0) == -1e10
    assert lib.orc_marginalise_over_position_shift(150.0) == pytest.approx(150 - np.log(D) - np.exp(-D))


def test_marginalise_posterior_against_scipy(lib):
    """cspline + QAG GK41 (marginalise_r.c) against scipy's natural CubicSpline and quad."""
    from radiolensfit2_gb300 import constants as K
    ro = np.array(K.ro_grid())[1:]
    rng = np.random.default_rng(1)
    for k in range(5):
        y = -0.5 * ((np.log(ro) - np.log(0.5 + 0.4 * k)) / 0.3) ** 2 * (1 + 3 * k) + rng.normal(0, 0.05, ro.size)
        yy = y.copy()
        got = lib.orc_marginalise_posterior_r(len(ro), O.dp(np.ascontiguousarray(ro)), O.dp(yy))
        ymax = max(y.max(), -10.0)
        cs = scipy_interp.CubicSpline(ro, y - ymax, bc_type="natural")
        val, _ = scipy_integrate.quad(lambda t: np.exp(cs(t)), ro[0], ro[-1], epsabs=0, epsrel=1e-10, limit=500)
        # QAG stops at epsrel 1e-3, so the reference itself is only that accurate
        assert got == pytest.approx(np.log(val) + ymax, abs=2e-3)


def test_mt19937_matches_reference_generator(lib):
    """gsl_rng_mt19937 seeding (init_genrand) and output: numpy's legacy RandomState uses the same
    Matsumoto-Nishimura generator and seeding for integer seeds."""
    lib.gsl_rng_alloc.restype = C.c_void_p
    lib.gsl_rng_alloc.argtypes = [C.c_void_p]
    lib.gsl_rng_set.argtypes = [C.c_void_p, C.c_ulong]
    lib.gsl_rng_get.restype = C.c_ulong
    lib.gsl_rng_get.argtypes = [C.c_void_p]
    lib.gsl_rng_free.argtypes = [C.c_void_p]
    T = C.c_void_p.in_dll(lib, "gsl_rng_mt19937")
    r = lib.gsl_rng_alloc(T)
    lib.gsl_rng_set(r, 12345)
    got = [lib.gsl_rng_get(r) for _ in range(1000)]
    lib.gsl_rng_free(r)
    want = np.random.RandomState(12345).randint(0, 2 ** 32, size=1000, dtype=np.uint64)
    assert got == [int(x) for x in want]
