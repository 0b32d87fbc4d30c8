"""The oracle's diffusion density against closed forms (CPU).

No fixture of the reference pins its diffusion likelihood, so the oracle's
Navarro-Fuss restatement is checked against the mathematics it states:
without variability the density at each boundary integrates to the Wiener
process's absorption probability, and the sv closed form equals numerical
integration over the drift distribution.
"""
import numpy as np
import pytest

integrate = pytest.importorskip("scipy.integrate")


def cv_of(a, v, z, sv=0.0, sz=0.0, st0=0.0, t0=0.0, d=0.0):
    row = [a, v, z, d, sz, sv, t0, st0]
    return np.array([row, row], float)


@pytest.mark.parametrize("a,v,z", [(1.0, 1.5, 0.5), (1.4, -0.8, 0.35), (0.8, 0.3, 0.6)])
def test_boundary_probabilities(oracle, a, v, z):
    cv = cv_of(a, v, z)
    lo = integrate.quad(lambda t: oracle.ddm_dens(t, cv, 0), 1e-6, 40, limit=400)[0]
    hi = integrate.quad(lambda t: oracle.ddm_dens(t, cv, 1), 1e-6, 40, limit=400)[0]
    x0 = z * a
    p_lower = (np.exp(-2 * v * a) - np.exp(-2 * v * x0)) / (np.exp(-2 * v * a) - 1)
    assert lo == pytest.approx(p_lower, abs=2e-6)
    assert hi == pytest.approx(1 - p_lower, abs=2e-6)


@pytest.mark.parametrize("t", [0.15, 0.4, 1.1])
def test_sv_closed_form_matches_drift_integral(oracle, t):
    a, v, z, sv = 1.2, 1.1, 0.45, 0.9
    want = integrate.quad(
        lambda u: oracle.ddm_dens(t, cv_of(a, u, z), 0) * np.exp(-0.5 * ((u - v) / sv) ** 2)
        / (sv * np.sqrt(2 * np.pi)), v - 10 * sv, v + 10 * sv, limit=200)[0]
    got = oracle.ddm_dens(t, cv_of(a, v, z, sv=sv), 0)
    assert got == pytest.approx(want, rel=1e-7)


def test_response_shift_and_floor(oracle):
    cv = cv_of(1.0, 1.0, 0.5, t0=0.3, d=0.1)
    # lower responses are shifted by t0 + d/2, upper by t0 - d/2
    assert oracle.ddm_dens(0.3 + 0.05 + 0.4, cv, 0) == pytest.approx(
        oracle.ddm_dens(0.4, cv_of(1.0, 1.0, 0.5), 0), rel=1e-14)
    assert oracle.ddm_dens(0.3 - 0.05 + 0.4, cv, 1) == pytest.approx(
        oracle.ddm_dens(0.4, cv_of(1.0, 1.0, 0.5), 1), rel=1e-14)
    assert oracle.ddm_dens(0.2, cv, 0) == 1e-10     # before the non-decision time
