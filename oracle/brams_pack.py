"""numpy restatement of BRAMS's column packing for the longwave solver and of
the heating-tendency write-back -- TEST INFRASTRUCTURE ONLY.

Follows ``radrrtmdrv`` in src/brams/radiate/rtm_driver.f90:
  * column order (j outer, i inner), :978-984;
  * surface temperature, emissivity, surface pressure, :990-1003;
  * layer pressure / temperature / vapour, cloud fields and radii, :1018-1043;
  * the extrapolated top level, :1045-1050;
  * layer and interface values, :1052-1076;
  * fixed trace gases and vapour volume mixing ratios, :1176-1231;
  * theta tendency and surface longwave flux out, :1443-1456;
  * the shortwave-only inputs (cosine of the zenith angle, albedos), :989,
    :992-996, and the surface shortwave flux out, :1448-1449.
BRAMS holds its fields and constants in default real (float32); the
statements mix them with real(8) exactly as below (each float32 operation is
rounded to float32 before it meets a double).  Ozone, aerosols and the
chemistry-coupled gas paths are the caller's (ozone climatology, CARMA):
they are not packed here.

The only importers are the tests; the product library never uses this file.
"""
from __future__ import annotations

import numpy as np

f4, f8 = np.float32, np.float64

# rconstants.f90:15-46 (default real) and mem_rrtm.f90:13-23 (real(8))
CP, RGAS, P00, STEFAN = f4(1004.0), f4(287.0), f4(1.0e5), f4(5.6696e-8)
CPOR = f4(CP / RGAS)
CPI = f4(f4(1.0) / CP)
ADJUST = 0.01
PMAR = 28.96
R_O3, R_CO2, R_CH4 = 1.0 / (47.998 / PMAR), 1.0 / (44.01 / PMAR), 1.0 / (16.04 / PMAR)
R_N2O, R_O2, R_H2O = 1.0 / (46.0055 / PMAR), 1.0 / (64.0 / PMAR), 1.0 / (18.01528 / PMAR)


def column_index(mxp, myp, ia, iz, ja, jz):
    """(i, j) zero-based of each packed column, j outer and i inner (:978-984)."""
    ii, jj = np.meshgrid(np.arange(ia - 1, iz), np.arange(ja - 1, jz), indexing="xy")
    return ii.ravel(), jj.ravel()


def pack_lw(f, ia, iz, ja, jz, iceflgsw=3, firsttime=False):
    """BRAMS fields f (float32; 3-D (mzp, mxp, myp), 2-D (mxp, myp); keys pi0,
    pp, theta, rv, cldf, lwl, iwl, rel, rei, rlongup, albedt) -> dict of the
    rrtmg_lw inputs, (ncol, nlay[+1]) float64 with nlay = mzp - 1."""
    mzp = f["pi0"].shape[0]
    nlay = mzp - 1
    i, j = column_index(f["pi0"].shape[1], f["pi0"].shape[2], ia, iz, ja, jz)
    n = i.size
    col = lambda a: a[:, i, j].T  # (ncol, mzp) float32
    pi0, pp, th, rv = col(f["pi0"]), col(f["pp"]), col(f["theta"]), col(f["rv"])
    out = {}
    # :990, :997 (not on the first call: emis stays 0 there), :1001-1003
    out["tsfc"] = f8(f4(f["rlongup"][i, j] / STEFAN)) ** 0.25
    emis = np.zeros((n, 16))
    if not firsttime:
        emis[:] = f8(f4(f4(1.0) - f["albedt"][i, j]))[:, None]
    out["emis"] = emis
    ps = f4(f4(f4(f4(f4(pi0[:, 0] + pp[:, 0]) + pi0[:, 1]) + pp[:, 1]) * CPI) * f4(0.5))
    psurf = (f8(P00) * f8(ps) ** f8(CPOR)) * ADJUST
    # :1018-1043 (k = 2..mzp -> index k-1 = 1..nlay, zero-based 0..nlay-1)
    picpi = f8(f4(f4(pi0[:, 1:] + pp[:, 1:]) * CPI))
    p = np.zeros((n, mzp))
    t = np.zeros((n, mzp))
    q = np.zeros((n, mzp))
    p[:, :nlay] = (f8(P00) * picpi ** f8(CPOR)) * ADJUST
    t[:, :nlay] = f8(th[:, 1:]) * picpi
    q[:, :nlay] = f8(rv[:, 1:])
    out["cldfrac"] = f8(col(f["cldf"])[:, 1:])
    out["clwp"] = f8(col(f["lwl"])[:, 1:])
    out["ciwp"] = f8(col(f["iwl"])[:, 1:])
    out["rel"] = f8(col(f["rel"])[:, 1:])
    rei = col(f["rei"])[:, 1:]
    if iceflgsw == 1:
        rei = np.minimum(f4(130.0), np.maximum(f4(13.0), rei))
    elif iceflgsw == 2:
        rei = np.minimum(f4(131.0), np.maximum(f4(5.0), rei))
    elif iceflgsw == 3:
        rei = np.minimum(f4(140.0), np.maximum(f4(5.0), f4(f4(f4(0.9021) * rei) - f4(7.0365))))
    else:
        rei = np.zeros_like(rei)  # the reference leaves reic at its initial 0
    out["rei"] = f8(rei)
    # :1045-1050 the extrapolated top level mzp (zero-based mzp-1)
    q[:, mzp - 1] = q[:, mzp - 2]
    p[:, mzp - 1] = p[:, mzp - 2] - 2.0 * (p[:, mzp - 2] - p[:, mzp - 3])
    t[:, mzp - 1] = t[:, mzp - 2] + (t[:, mzp - 2] - t[:, mzp - 3]) / (p[:, mzp - 2] - p[:, mzp - 3]) * (
        p[:, mzp - 1] - p[:, mzp - 2])
    # :1052-1076
    play, tlay = p[:, :nlay].copy(), t[:, :nlay].copy()
    plev = np.zeros((n, nlay + 1))
    tlev = np.zeros((n, nlay + 1))
    plev[:, 1:nlay] = (p[:, 1:nlay] + p[:, 0:nlay - 1]) * 0.5
    tlev[:, 1:nlay] = (t[:, 1:nlay] + t[:, 0:nlay - 1]) * 0.5
    plev[:, 0] = psurf
    a = f4(f4(th[:, 0] * f4(pi0[:, 0] + pp[:, 0])) * CPI)
    b = f4(f4(th[:, 1] * f4(pi0[:, 1] + pp[:, 1])) * CPI)
    tlev[:, 0] = f8(f4(f4(0.5) * f4(a + b)))
    plev[:, nlay] = plev[:, nlay - 1] - 2.0 * (plev[:, nlay - 1] - play[:, nlay - 1])
    tlev[:, nlay] = tlev[:, nlay - 1] + (tlev[:, nlay - 1] - tlev[:, nlay - 2]) / (
        plev[:, nlay - 1] - plev[:, nlay - 2]) * (plev[:, nlay] - plev[:, nlay - 1])
    out.update(play=play, tlay=tlay, plev=plev, tlev=tlev)
    # :1224 (vapour of layer k-1 from q at k), fixed gases :1176-1231
    out["h2ovmr"] = q[:, 1:mzp] * R_H2O
    full = lambda v: np.full((n, nlay), v)
    out["co2vmr"] = full(f8(f4(379.0e-6)) * R_CO2)
    out["ch4vmr"] = full(f8(f4(1774.0e-9)) * R_CH4)
    out["n2ovmr"] = full(f8(f4(319.0e-9)) * R_N2O)
    out["o2vmr"] = full(f8(f4(0.209488)) * R_O2)
    out["cfc11vmr"] = full(f8(f4(0.251e-9)))
    out["cfc12vmr"] = full(f8(f4(0.538e-9)))
    out["cfc22vmr"] = full(f8(f4(0.169e-9)))
    out["ccl4vmr"] = full(f8(f4(0.093e-9)))
    return out


def unpack_lw(hr, dflx, swhr, mzp, mxp, myp, ia, iz, ja, jz, fthrd=None, rlong=None):
    """Theta tendency (K/s) and surface downward longwave flux into BRAMS's
    float32 fields (:1443-1456); hr, swhr (ncol, >= nlay), dflx (ncol, >= 1)
    float64.  Columns outside the packed range keep fthrd/rlong as given."""
    fthrd = np.zeros((mzp, mxp, myp), np.float32) if fthrd is None else fthrd.copy()
    rlong = np.zeros((mxp, myp), np.float32) if rlong is None else rlong.copy()
    i, j = column_index(mxp, myp, ia, iz, ja, jz)
    rlong[i, j] = f4(dflx[:, 0])
    sw = swhr if swhr is not None else np.zeros_like(hr)
    v = f4((sw[:, 0:mzp - 2] + hr[:, 0:mzp - 2]) / f8(f4(86400.0)))  # k = 2..mzp-1
    fthrd[1:mzp - 1, i, j] = v.T
    fthrd[0, i, j] = fthrd[1, i, j]
    fthrd[mzp - 1, i, j] = fthrd[mzp - 2, i, j]
    return fthrd, rlong


def pack_sw(cosz, albedt, ia, iz, ja, jz, firsttime=False):
    """BRAMS's cosz and albedt (float32 (mxp, myp)) -> coszen and the four
    albedos of rrtmg_sw (ncol,) float64 (:989, :992-996; the albedos keep the
    0 they are allocated with on the first call, :933-936)."""
    i, j = column_index(cosz.shape[0], cosz.shape[1], ia, iz, ja, jz)
    out = {"coszen": f8(cosz[i, j])}
    al = np.zeros(i.size) if firsttime else f8(albedt[i, j])
    for k in ("asdir", "aldir", "asdif", "aldif"):
        out[k] = al.copy()
    return out


def unpack_sw(swdflx, mxp, myp, ia, iz, ja, jz, rshort=None):
    """The surface downward shortwave flux into BRAMS's float32 rshort
    (:1448-1449): 0 where swdflx(:, 1) < 0.5.  Columns outside the packed
    range keep rshort as given."""
    rshort = np.zeros((mxp, myp), np.float32) if rshort is None else rshort.copy()
    i, j = column_index(mxp, myp, ia, iz, ja, jz)
    v = swdflx[:, 0]
    rshort[i, j] = np.where(v < 0.5, f4(0.0), f4(v))
    return rshort
