"""The shortwave fp32 kernel evaluates reftra_sw (rrtmg_sw_reftra.f90:107-326,
kmodts = 2) in a rearranged form: the direct-beam reflectance and
transmittance have a removable singularity at k mu0 = 1, which the kernel
divides out, leaving q = (e1 - e2) / (1 - k mu0) with e1 = exp(-k tau),
e2 = exp(-tau / mu0), and k is formed from the co-albedo as
sqrt(2 (1 - w) (gamma1 + gamma2)).  These are identities of the reference's
formulas; this test states both forms in fp64 (numpy) on random layers and
checks that they agree, including the exact Taylor-range divided difference
q = x2 (1 - (x1 + x2) / 2) the kernel uses where both exponents are below
od_lo = 0.06 (there the reference takes exp(-x) = 1 - x + x^2 / 2)."""
import numpy as np


def _gammas(zg, zw, mu):
    g3 = 3.0 * zg
    g1 = (8.0 - zw * (5.0 + g3)) * 0.25
    g2 = 3.0 * (zw * (1.0 - zg)) * 0.25
    g3_ = (2.0 - g3 * mu) * 0.25
    return g1, g2, g3_, 1.0 - g3_


def _reference(zg, zw, mu, tau, e1, e2):
    """rrtmg_sw_reftra.f90:246-282 as written (given the two exponentials)."""
    g1, g2, g3, g4 = _gammas(zg, zw, mu)
    a1 = g1 * g4 + g2 * g3
    a2 = g1 * g3 + g2 * g4
    k = np.sqrt(g1 * g1 - g2 * g2)
    p = k * mu
    rp1, rm1, k2, rpp, kg = 1.0 + p, 1.0 - p, 2.0 * k, 1.0 - p * p, k + g1
    r1, r2, r3 = rm1 * (a2 + k * g3), rp1 * (a2 - k * g3), k2 * (g3 - a2 * mu)
    r4, r5 = rpp * kg, rpp * (k - g1)
    t1, t2, t3 = rp1 * (a1 + k * g4), rm1 * (a1 - k * g4), k2 * (g4 + a1 * mu)
    ep1, ep2 = 1.0 / e1, 1.0 / e2
    den = r4 * ep1 + r5 * e1
    pref = zw * (r1 * ep1 - r2 * e1 - r3 * e2) / den
    ptra = e2 - e2 * zw * (t1 * ep1 - t2 * e1 - t3 * ep2) / den
    return pref, ptra


def _rearranged(zg, zw, mu, tau, e1, e2, q):
    """The kernel's form (sw_kernel.cuh reftra_f), q = (e1 - e2) / (1 - k mu)."""
    g1, g2, g3, g4 = _gammas(zg, zw, mu)
    co = 1.0 - zw
    k = np.sqrt(2.0 * co * (g1 + g2))
    p = k * mu
    a1, a2 = g1 * g4 + g2 * g3, g1 * g3 + g2 * g4
    kg = k + g1
    dn = kg + (k - g1) * e1 * e1
    uo = (1.0 - e1 * e2) / (1.0 + p)
    a, b, c, d = a2, k * g3, a1, k * g4
    pref = zw * ((a + b) * uo - (a - b) * e1 * q) / dn
    ptra = e2 - zw * ((c - d) * e1 * uo - (c + d) * q) / dn
    return pref, ptra


def test_rearranged_reftra_equals_the_reference():
    rng = np.random.default_rng(11)
    n = 20000
    zg = rng.uniform(0.0, 0.9, n)
    zw = np.where(rng.uniform(size=n) < 0.5, rng.uniform(0.0, 0.99, n), 1.0 - 10.0 ** rng.uniform(-5, -1, n))
    mu = rng.uniform(0.05, 1.0, n)
    tau = 10.0 ** rng.uniform(-3, 1.5, n)
    g1, g2, _, _ = _gammas(zg, zw, mu)
    k = np.sqrt(g1 * g1 - g2 * g2)
    p = k * mu
    keep = np.abs(1.0 - p) > 1e-3  # away from the singularity, where both forms are well conditioned in fp64
    zg, zw, mu, tau, k, p = zg[keep], zw[keep], mu[keep], tau[keep], k[keep], p[keep]
    e1, e2 = np.exp(-k * tau), np.exp(-tau / mu)
    want_r, want_t = _reference(zg, zw, mu, tau, e1, e2)
    got_r, got_t = _rearranged(zg, zw, mu, tau, e1, e2, (e1 - e2) / (1.0 - p))
    assert np.abs(got_r - want_r).max() <= 1e-9 * (1.0 + np.abs(want_r).max())
    assert np.abs(got_t - want_t).max() <= 1e-9 * (1.0 + np.abs(want_t).max())


def test_taylor_range_divided_difference_is_exact():
    """Both exponents below 0.06: with the reference's expansion exp(-x) =
    1 - x + x^2/2, (e1 - e2) / (1 - k mu) = x2 (1 - (x1 + x2) / 2) exactly,
    x1 = k tau, x2 = tau / mu (so x1 = k mu x2)."""
    rng = np.random.default_rng(5)
    x2 = rng.uniform(1e-6, 0.06, 5000)
    kmu = rng.uniform(0.5, 1.5, 5000)
    kmu = kmu[np.abs(1.0 - kmu) > 1e-4]
    x2 = x2[: kmu.size]
    x1 = kmu * x2
    ok = x1 <= 0.06
    x1, x2, kmu = x1[ok], x2[ok], kmu[ok]
    e1 = 1.0 - x1 + 0.5 * x1 * x1
    e2 = 1.0 - x2 + 0.5 * x2 * x2
    q = (e1 - e2) / (1.0 - kmu)
    assert np.abs(q - x2 * (1.0 - 0.5 * (x1 + x2))).max() <= 1e-9 * np.abs(q).max()


def test_conservative_test_on_the_co_albedo():
    """zwo = zw / (1 - (1 - zw) q^2) >= zwcrit holds exactly when
    (1 - zw)(1 - q^2) <= (1 - zwcrit) (1 - (1 - zw) q^2) for a positive
    denominator, q = zg / (1 - zg) (rrtmg_sw_reftra.f90:140-147)."""
    rng = np.random.default_rng(3)
    zg = rng.uniform(0.0, 0.95, 20000)
    co = 10.0 ** rng.uniform(-9, -1, 20000)
    zw = 1.0 - co
    q2 = (zg / (1.0 - zg)) ** 2
    den = 1.0 - co * q2
    zwcrit = 0.9999995
    ref = (den != 0) & (zw / den >= zwcrit)
    got = (den > 0) & (co * (1.0 - q2) <= (1.0 - zwcrit) * den)
    close = np.abs(zw / den - zwcrit) < 1e-12  # rounding ties of the two forms
    assert np.array_equal(ref[~close], got[~close])
