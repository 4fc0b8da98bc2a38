"""Seeded BRAMS-like model fields for the column-packing tests: a hydrostatic
atmosphere on BRAMS's staggered thermodynamic levels (level 1 below the
surface), Exner function split into reference and perturbation parts,
vapour, cloud fraction and water paths, radii, and surface fields, all in
BRAMS's default-real (float32) Fortran-ordered arrays."""
import numpy as np

CP, RGAS, P00, STEFAN = 1004.0, 287.0, 1.0e5, 5.6696e-8


def brams_fields(mzp: int, mxp: int, myp: int, seed: int, dz: float = 400.0) -> dict:
    rs = np.random.default_rng(seed)
    z = (np.arange(mzp) - 0.5) * dz                               # level 1 (index 0) is below ground
    ps = rs.uniform(95000.0, 102000.0, (mxp, myp))
    ts = rs.uniform(280.0, 302.0, (mxp, myp))
    p = ps[None] * np.exp(-z[:, None, None] / 8000.0)
    t = np.maximum(ts[None] - 6.5e-3 * z[:, None, None], 212.0) + rs.normal(0.0, 0.5, (mzp, mxp, myp))
    exner = CP * (p / P00) ** (RGAS / CP)
    pp = rs.normal(0.0, 0.3, (mzp, mxp, myp))
    rv = 0.012 * np.exp(-np.maximum(z, 0.0)[:, None, None] / 2500.0) * rs.lognormal(0.0, 0.2, (mzp, mxp, myp))
    cloudy = (rs.random((mzp, mxp, myp)) < 0.3) & (np.arange(mzp)[:, None, None] >= 2) & (
        np.arange(mzp)[:, None, None] < min(mzp - 1, 24))
    cldf = np.where(cloudy, rs.uniform(0.05, 1.0, (mzp, mxp, myp)), 0.0)
    lwl = np.where(cloudy & (t > 253.0), rs.lognormal(np.log(50.0), 0.8, (mzp, mxp, myp)), 0.0)
    iwl = np.where(cloudy & (t < 263.0), rs.lognormal(np.log(20.0), 0.8, (mzp, mxp, myp)), 0.0)
    F = lambda a: np.asfortranarray(np.asarray(a, dtype=np.float32))
    return {
        "pi0": F(exner - pp), "pp": F(pp), "theta": F(t * CP / exner), "rv": F(rv),
        "cldf": F(cldf), "lwl": F(lwl), "iwl": F(iwl),
        "rel": F(rs.uniform(5.0, 20.0, (mzp, mxp, myp))), "rei": F(rs.uniform(20.0, 120.0, (mzp, mxp, myp))),
        "rlongup": F(STEFAN * ts ** 4), "albedt": F(rs.uniform(0.02, 0.1, (mxp, myp))),
    }


def ozone(play: np.ndarray) -> np.ndarray:
    """A fixed ozone profile (volume mixing ratio) on the packed layers: a
    peak of 8 ppmv near 30 hPa (stands in for the driver's climatology)."""
    return np.asfortranarray(8.0e-6 * np.exp(-np.log(play / 30.0) ** 2 / 2.0) + 2.0e-8)
