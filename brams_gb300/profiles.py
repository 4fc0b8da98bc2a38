"""Seeded synthetic column inputs in the rrtmg_lw argument layout.

The reference drives ``rrtmg_lw`` from BRAMS model state
(``src/brams/radiate/rtm_driver.f90:980-1231``).  For benchmarking and parity
this module builds the same argument arrays from an idealised, seeded
atmosphere instead:

* pressure levels log-spaced from 1000 hPa to ``ptop``; layer pressures at the
  log-midpoints (``plev(:,1)`` is the surface, as in the reference);
* temperature 288 K at the surface with a 6.5 K/km lapse rate down to a
  217 K isothermal stratosphere; heights from the hypsometric equation;
  layer temperatures carry N(0, ``t_noise``) noise;
* H2O vmr 0.015*exp(-z/2.5 km) times lognormal(0, ``h2o_sigma``);
* O3 a Gaussian of 8 ppmv peak at 25 km, width 6 km;
* CO2 400 ppmv, CH4 1.8 ppmv, N2O 0.32 ppmv, O2 and CFCs at the constant
  values the BRAMS driver uses (``rtm_driver.f90:1218,1228-1231``, default
  real literals, hence rounded through float32);
* clouds in layers 5-20 with probability 0.3, fraction U(0,1), water path
  lognormal with mean 50 g m-2 and sigma 0.8, ice where T < 253 K and liquid
  elsewhere; liquid radius 10 um, ice generalised size 50 um;
* surface emissivity U(0.95, 1.0) in all 16 bands, zero aerosol.

Random numbers come from a counter-based SplitMix64 stream (pure integer
arithmetic), so the same seed gives the same uniforms on any platform.
All 2-D arrays are returned Fortran-ordered with shape (ncol, nlay[+1]).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix(counter: np.ndarray) -> np.ndarray:
    z = counter.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


class Stream:
    """Counter-based uniform/normal generator: draw k of stream s is a pure function."""

    def __init__(self, seed: int):
        self.base = np.uint64(seed & 0xFFFFFFFF) << np.uint64(32)
        self.pos = 0

    def uniform(self, shape) -> np.ndarray:
        n = int(np.prod(shape))
        with np.errstate(over="ignore"):
            ctr = self.base + np.arange(self.pos, self.pos + n, dtype=np.uint64)
            bits = _splitmix(ctr)
        self.pos += n
        u = ((bits >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)
        return u.reshape(shape, order="F")

    def normal(self, shape) -> np.ndarray:
        u1 = self.uniform(shape)
        u2 = self.uniform(shape)
        return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


O2_VMR = float(np.float32(0.209488))
CFC11 = float(np.float32(0.251e-9))
CFC12 = float(np.float32(0.538e-9))
CFC22 = float(np.float32(0.169e-9))
CCL4 = float(np.float32(0.093e-9))


@dataclass
class ProfileSpec:
    ncol: int
    nlay: int
    seed: int = 20240601
    ptop: float = 10.0
    t_noise: float = 2.0
    h2o_sigma: float = 0.3
    cloud_layers: tuple = (5, 20)
    cloud_prob: float = 0.3
    rel: float = 10.0
    rei: float = 50.0
    extra: dict = field(default_factory=dict)


def base_profile(nlay: int, ptop: float):
    """Smooth (noise-free) levels: plev, play, tlev, z at levels and layer midpoints."""
    plev = 1000.0 * (ptop / 1000.0) ** (np.arange(nlay + 1) / nlay)
    play = np.sqrt(plev[:-1] * plev[1:])
    rd, g = 287.04, 9.80665

    def tz(zkm):
        return np.maximum(288.0 - 6.5 * zkm, 217.0)

    z = np.zeros(nlay + 1)
    for k in range(nlay):
        t0 = tz(z[k])
        dz = rd * t0 / g * np.log(plev[k] / plev[k + 1]) / 1000.0
        t1 = tz(z[k] + dz)
        z[k + 1] = z[k] + rd * 0.5 * (t0 + t1) / g * np.log(plev[k] / plev[k + 1]) / 1000.0
    zmid = np.zeros(nlay)
    for k in range(nlay):
        t0 = tz(z[k])
        zmid[k] = z[k] + rd * t0 / g * np.log(plev[k] / play[k]) / 1000.0
    return plev, play, tz(z), tz(zmid), z, zmid


def make_state(spec: ProfileSpec) -> dict:
    """Column state and layer cloud properties (before McICA sub-columns)."""
    ncol, nlay = spec.ncol, spec.nlay
    rs = Stream(spec.seed)
    plev1, play1, tlev1, tlay1, z1, zmid = base_profile(nlay, spec.ptop)
    F = lambda a: np.asfortranarray(a)
    out = {}
    out["plev"] = F(np.tile(plev1, (ncol, 1)))
    out["play"] = F(np.tile(play1, (ncol, 1)))
    out["tlev"] = F(np.tile(tlev1, (ncol, 1)))
    tlay = np.tile(tlay1, (ncol, 1)) + spec.t_noise * rs.normal((ncol, nlay))
    out["tlay"] = F(tlay)
    out["tsfc"] = tlev1[0] + 1.0 * rs.normal((ncol,))
    h2o = 0.015 * np.exp(-zmid / 2.5)[None, :] * np.exp(spec.h2o_sigma * rs.normal((ncol, nlay)))
    out["h2ovmr"] = F(np.clip(h2o, 3.0e-6, 0.05))
    o3 = 8.0e-6 * np.exp(-0.5 * ((zmid - 25.0) / 6.0) ** 2) + 2.0e-8
    out["o3vmr"] = F(np.tile(o3, (ncol, 1)))
    const = lambda v: F(np.full((ncol, nlay), v))
    out["co2vmr"] = const(400.0e-6)
    out["ch4vmr"] = const(1.8e-6)
    out["n2ovmr"] = const(0.32e-6)
    out["o2vmr"] = const(O2_VMR)
    out["cfc11vmr"] = const(CFC11)
    out["cfc12vmr"] = const(CFC12)
    out["cfc22vmr"] = const(CFC22)
    out["ccl4vmr"] = const(CCL4)
    out["emis"] = F(0.95 + 0.05 * rs.uniform((ncol, 16)))
    # layer clouds
    l0, l1 = spec.cloud_layers
    present = rs.uniform((ncol, nlay)) < spec.cloud_prob
    mask = np.zeros((ncol, nlay), dtype=bool)
    mask[:, l0 - 1:min(l1, nlay)] = True
    present &= mask
    frac = rs.uniform((ncol, nlay))
    mu = np.log(50.0) - 0.5 * 0.8 ** 2
    wp = np.exp(mu + 0.8 * rs.normal((ncol, nlay)))
    cold = tlay < 253.0
    out["cldfrac"] = F(np.where(present, frac, 0.0))
    out["ciwp"] = F(np.where(present & cold, wp, 0.0))
    out["clwp"] = F(np.where(present & ~cold, wp, 0.0))
    out["rei"] = F(np.full((ncol, nlay), spec.rei))
    out["rel"] = F(np.full((ncol, nlay), spec.rel))
    out["tauaer"] = np.zeros((ncol, nlay, 16), order="F")
    return out


WORKLOADS = {
    # name: (ncol, nlay, ptop, t_noise, h2o_sigma)
    "oracle_64x64x38": dict(ncol=64 * 64, nlay=38, ptop=10.0, t_noise=2.0, h2o_sigma=0.3),
    "drop_in_360x300x45": dict(ncol=360 * 300, nlay=45, ptop=10.0, t_noise=4.0, h2o_sigma=0.5),
    "eval_512x512x45": dict(ncol=512 * 512, nlay=45, ptop=10.0, t_noise=4.0, h2o_sigma=0.5),
    "scale_2048x1024x4x60": dict(ncol=2048 * 1024 * 4, nlay=60, ptop=5.0, t_noise=4.0, h2o_sigma=0.5),
}


def workload_spec(name: str, ncol: int | None = None, seed: int = 20240601) -> ProfileSpec:
    c = dict(WORKLOADS[name])
    if ncol is not None:
        c["ncol"] = ncol
    return ProfileSpec(seed=seed, **c)
