"""CPU mirror of the device p-value arithmetic of the Gaussian pmax kernels
(gpucsl_gb300/csrc/gauss.cu: sf_table_build, two_sf_tab, fisher_z), checked against
scipy: the Taylor-table erfc and the atanh series must agree with the library values
far inside the 1e-9 relative pmax tolerance.  The mirror repeats the same operation
order in FP64 numpy."""
import math

import numpy as np
import pytest

SF_CENTRES, SF_TERMS = 32, 13


def sf_table():
    a = np.zeros((SF_CENTRES, SF_TERMS))
    for m in range(SF_CENTRES):
        c = (m + 0.5) * 0.125
        bprev, b = 0.0, -1.12837916709551257390 * math.exp(-c * c)
        a[m, 0] = math.erfc(c)
        for k in range(SF_TERMS - 1):
            a[m, k + 1] = b / (k + 1)
            bn = (-2.0 * c * b - 2.0 * bprev) / (k + 1)
            bprev, b = b, bn
    return a


def two_sf_tab(z, a):
    x = abs(z) * 0.70710678118654752440
    if not x < 4.0:
        return math.erfc(x)
    m = int(x * 8.0)
    t = x - (m + 0.5) * 0.125
    v = a[m, SF_TERMS - 1]
    for k in range(SF_TERMS - 2, -1, -1):
        v = v * t + a[m, k]
    return v


def fisher_z(r):
    u = r * r
    if u < 0.01:
        s = 1.0 / 19.0
        for d in (17, 15, 13, 11, 9, 7, 5, 3):
            s = s * u + 1.0 / d
        s = s * u + 1.0
        return abs(r) * s
    return abs(0.5 * math.log(abs((1.0 + r) / (1.0 - r))))


def test_taylor_erfc_matches_scipy():
    sc = pytest.importorskip("scipy.stats")
    a = sf_table()
    z = np.concatenate([np.linspace(0, 6.0, 20001), [1e-12, 5.6568542494923806, 5.6568542494923797]])
    got = np.array([two_sf_tab(v, a) for v in z])
    ref = 2.0 * sc.norm.sf(z)
    rel = np.abs(got - ref) / ref
    assert rel.max() < 1e-13, float(rel.max())


def test_atanh_series_matches_log_form():
    r = np.concatenate([np.linspace(-0.0999, 0.0999, 4001), [1e-300, -1e-8, 0.09999999]])
    got = np.array([fisher_z(v) for v in r])
    ref = np.abs(np.arctanh(r))
    nz = ref > 0
    assert (np.abs(got[nz] - ref[nz]) / ref[nz]).max() < 1e-14
    # the pmax it feeds: 2 sf(sqrt(n - 3) Z) within 1e-12 relative of the log form
    sc = pytest.importorskip("scipy.stats")
    for n in (20, 1000, 10000, 100000):
        zl = np.array([abs(0.5 * math.log(abs((1 + v) / (1 - v)))) for v in r])
        p_ser = 2 * sc.norm.sf(math.sqrt(n - 3) * got)
        p_log = 2 * sc.norm.sf(math.sqrt(n - 3) * zl)
        assert (np.abs(p_ser - p_log) / p_log).max() < 1e-10
