"""GPU gas optics band by band: taut and Planck fractions of the column
kernel against the oracle's taumol (rrtmg_lw_taumol.f90) plus aerosol add."""
import numpy as np
import pytest

import pyoracle
from brams_gb300.profiles import ProfileSpec, make_state

pytestmark = pytest.mark.gpu

NGS0 = [0, 10, 22, 38, 52, 68, 76, 88, 96, 108, 114, 122, 130, 134, 136, 138, 140]


@pytest.mark.parametrize("nlay,ptop", [(38, 10.0), (60, 5.0)])
def test_taumol_bands(ctx, nlay, ptop):
    st = make_state(ProfileSpec(ncol=8, nlay=nlay, seed=31, ptop=ptop, t_noise=8.0, h2o_sigma=0.8))
    st["tauaer"] = np.asfortranarray(np.random.default_rng(0).uniform(0, 0.05, (8, nlay, 16)))
    taut, fracs = ctx.gas_optics_diag(st)
    mc0 = {k: np.zeros((140, 8, nlay), order="F") for k in ("cldfmcl", "taucmcl", "ciwpmcl", "clwpmcl")}
    mc0["reicmcl"] = np.asfortranarray(st["rei"])
    mc0["relqmcl"] = np.asfortranarray(st["rel"])
    worst = {}
    for icol in range(8):
        im = pyoracle.column_intermediates(st, mc0, icol + 1, icld=0)
        rt, rf = im["taut"], im["fracs"]
        gt, gf = taut[icol].astype(np.float64), fracs[icol].astype(np.float64)
        for b in range(16):
            g0, g1 = NGS0[b], NGS0[b + 1]
            et = np.abs(gt[:, g0:g1] - rt[:, g0:g1]) / (np.abs(rt[:, g0:g1]) + 1e-6)
            ef = np.abs(gf[:, g0:g1] - rf[:, g0:g1])
            worst[b + 1] = max(worst.get(b + 1, 0.0), float(et.max()), float(ef.max()))
    bad = {b: e for b, e in worst.items() if e > 2e-4}
    assert not bad, f"bands with relative taut/frac error > 2e-4: {bad}"
