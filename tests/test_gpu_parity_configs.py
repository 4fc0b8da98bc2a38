"""GPU parity on the benchmark configurations and across the cloud-optics options.

* the 64x64x38 oracle configuration in full (4,096 columns);
* 8,192 columns of the 360x300x45 operational-scale generator;
* every ice/liquid optics option of cldprmc (rrtmg_lw_cldprmc.f90:197-266)
  with particle sizes drawn across each option's valid range, and a nonzero
  aerosol optical depth -- through gb_rrtmg_lw against the FP64 oracle.

Tolerances: fluxes within 0.05 W m-2, heating rates within 0.01 K/day,
surface-temperature derivatives within 1e-3 W m-2 K-1.
"""
import numpy as np
import pytest

import pyoracle
from brams_gb300.profiles import ProfileSpec, make_state, workload_spec

pytestmark = pytest.mark.gpu

FLUX_TOL, HR_TOL, DER_TOL = 0.05, 0.01, 1e-3


def _assert_parity(out, ref):
    for k in ("uflx", "dflx", "uflxc", "dflxc"):
        assert np.abs(out[k] - ref[k]).max() <= FLUX_TOL, (k, float(np.abs(out[k] - ref[k]).max()))
    for k in ("hr", "hrc"):
        assert np.abs(out[k] - ref[k]).max() <= HR_TOL, (k, float(np.abs(out[k] - ref[k]).max()))
    for k in ("duflx_dt", "duflxc_dt"):
        assert np.abs(out[k] - ref[k]).max() <= DER_TOL, (k, float(np.abs(out[k] - ref[k]).max()))


def _run(ctx, st, seed, **flags):
    tauc = pyoracle.cldprop_columns(st, inflag=flags.get("inflglw", 2), iceflag=flags.get("iceflglw", 3),
                                    liqflag=flags.get("liqflglw", 1))
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=seed)
    ref = pyoracle.rrtmg_lw(st, mc, nthreads=16, **flags)
    out = ctx.rrtmg_lw(st, mc, **flags)
    return out, ref


def test_config1_in_full(ctx):
    st = make_state(workload_spec("oracle_64x64x38"))
    assert st["play"].shape == (4096, 38)
    out, ref = _run(ctx, st, seed=1)
    _assert_parity(out, ref)


def test_config2_sample(ctx):
    st = make_state(workload_spec("drop_in_360x300x45", ncol=8192))
    assert st["play"].shape == (8192, 45)
    out, ref = _run(ctx, st, seed=1)
    _assert_parity(out, ref)


# valid particle sizes per option (cldprmc.f90:217-266): ice radius or
# generalised size by iceflag, liquid radius for liqflag 1
ICE_RANGE = {0: (10.0, 140.0), 1: (13.0, 130.0), 2: (5.0, 131.0), 3: (5.0, 140.0)}
LIQ_RANGE = {0: (2.5, 60.0), 1: (2.5, 60.0)}


@pytest.mark.parametrize("iceflag", [0, 1, 2, 3])
@pytest.mark.parametrize("liqflag", [0, 1])
def test_cloud_optics_options_and_radii(ctx, iceflag, liqflag):
    st = make_state(ProfileSpec(ncol=96, nlay=45, seed=300 + 10 * iceflag + liqflag, t_noise=4.0, h2o_sigma=0.5,
                                cloud_prob=0.6))
    rng = np.random.default_rng(7 + iceflag + 4 * liqflag)
    lo, hi = ICE_RANGE[iceflag]
    st["rei"] = np.asfortranarray(rng.uniform(lo, hi, st["rei"].shape))
    lo, hi = LIQ_RANGE[liqflag]
    st["rel"] = np.asfortranarray(rng.uniform(lo, hi, st["rel"].shape))
    st["tauaer"] = np.asfortranarray(rng.uniform(0.0, 0.05, st["tauaer"].shape))
    # both phases present somewhere: mixed-phase layers near the freezing level
    mixed = (st["cldfrac"] > 0) & (st["tlay"] > 245.0) & (st["tlay"] < 262.0)
    st["ciwp"] = np.asfortranarray(np.where(mixed, 0.5 * (st["ciwp"] + st["clwp"]) + 1.0, st["ciwp"]))
    st["clwp"] = np.asfortranarray(np.where(mixed, st["ciwp"], st["clwp"]))
    assert (st["ciwp"] > 0).any() and (st["clwp"] > 0).any()
    out, ref = _run(ctx, st, seed=11, iceflglw=iceflag, liqflglw=liqflag)
    _assert_parity(out, ref)
    # the clouds matter: the all-sky and clear-sky fluxes differ
    assert np.abs(out["dflx"] - out["dflxc"]).max() > 1.0
