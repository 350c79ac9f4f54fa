"""CPU: the identities behind the J/E tables of the mixed form's full
assembly (k_cheb_build_je, k_assemble_je_df), checked with SciPy's Bessel
functions at complex arguments:

* the ascending-series forms of the entire parts
    G0 = Y0 - l J0 = (2/pi) [(ln(k/2) + gamma) J0 - s0],
    G1 = Y1 - l J1 + 2/(pi z) = (2/pi)(ln(k/2) + gamma) J1 - s1 / pi,
  z = k r, l = (2/pi) ln r (A&S 9.1.11, 9.1.13), for |z| < 4;
* the recombination of the tabulated series P = kaL2 J1, U = kaL2 (J1 + i G1),
  R = kd J0, W = kd (J0 + i G0) into the four kernel terms:
  kaL2 H1 = U + i l P + 1/(pi r), kd H0 = W + i l R, kaL1 J1 = (i/pi) P,
  kg J0 = (i/pi) R, with kaL1 = -k/2pi, kaL2 = ik/2, kg = -ik/2pi, kd = -k/2."""
import numpy as np
import pytest

sp = pytest.importorskip("scipy.special")
GAMMA = 0.57721566490153286061


def _series(k, r):
    z = k * r
    h = 0.5 * z
    q = -h * h
    t0, t1 = 1.0 + 0j, h
    a0 = a1 = s0 = s1 = 0j
    hm = 0.0
    for m in range(48):
        if m > 0:
            t0 = t0 * q / (m * m)
            t1 = t1 * q / (m * (m + 1))
            hm += 1.0 / m
        a0 += t0
        a1 += t1
        s0 += hm * t0
        s1 += (2 * hm + 1.0 / (m + 1)) * t1
        if abs(t0) < 1e-18 and abs(t1) < 1e-18:
            break
    lkg = np.log(0.5 * k) + GAMMA
    return a0, a1, (2 / np.pi) * (lkg * a0 - s0), (2 / np.pi) * lkg * a1 - s1 / np.pi


@pytest.mark.parametrize("k", [200.0 + 0.4j, 25.0 - 0.3j, 2.0 + 0.1j, 60.0 + 0.0j])
def test_entire_parts_series(k):
    rng = np.random.default_rng(7)
    for r in rng.uniform(1e-6, 3.9 / abs(k), 40):
        z = k * r
        l = (2 / np.pi) * np.log(r)
        j0, j1, g0, g1 = _series(k, r)
        J0, J1, Y0, Y1 = sp.jv(0, z), sp.jv(1, z), sp.yv(0, z), sp.yv(1, z)
        assert abs(j0 - J0) <= 1e-15 * max(1.0, abs(J0))
        assert abs(j1 - J1) <= 1e-15 * max(1.0, abs(J1))
        # the SciPy side cancels: its error is a few eps times the sum of the
        # magnitudes of its terms (|Y1| ~ 2/(pi z) is large at small z)
        e0 = 1e-15 * (1.0 + abs(Y0) + abs(l * J0))
        e1 = 1e-15 * (1.0 + abs(Y1) + abs(l * J1) + 2 / abs(np.pi * z))
        assert abs(g0 - (Y0 - l * J0)) <= e0
        assert abs(g1 - (Y1 - l * J1 + 2 / (np.pi * z))) <= e1


@pytest.mark.parametrize("k", [200.0 + 0.4j, 25.0 - 0.3j])
def test_recombination(k):
    kaL1, kaL2, kg, kd = -k / (2 * np.pi), 0.5j * k, -1j * k / (2 * np.pi), -0.5 * k
    for r in [1e-3, 0.01, 0.3, 2.2]:
        z = k * r
        l = (2 / np.pi) * np.log(r)
        J0, J1, Y0, Y1 = sp.jv(0, z), sp.jv(1, z), sp.yv(0, z), sp.yv(1, z)
        g0, g1 = Y0 - l * J0, Y1 - l * J1 + 2 / (np.pi * z)
        P, U, R, W = kaL2 * J1, kaL2 * (J1 + 1j * g1), kd * J0, kd * (J0 + 1j * g0)
        H0, H1 = sp.hankel1(0, z), sp.hankel1(1, z)
        sc = abs(k) * max(1.0, abs(H1))
        assert abs((U + 1j * l * P + 1 / (np.pi * r)) - kaL2 * H1) <= 1e-13 * sc
        assert abs((W + 1j * l * R) - kd * H0) <= 1e-13 * sc
        assert abs(1j / np.pi * P - kaL1 * J1) <= 1e-14 * sc
        assert abs(1j / np.pi * R - kg * J0) <= 1e-14 * sc
