"""Several contexts on one device.  The kernels' constant table blocks exist
once per device, so the contexts of a device must agree on the tables (table
files and cpdair): a second context with the same tables solves to the same
bits, one with a different cpdair is refused (GB_LW_E_TABLES) and leaves the
live context's results unchanged, in the longwave and the shortwave."""
import numpy as np
import pytest

import pyoracle
from brams_gb300 import rrtmg_lw as R
from brams_gb300.profiles import ProfileSpec, make_state

pytestmark = pytest.mark.gpu
GB_LW_E_TABLES = -3  # include/gb_rrtmg_lw.h


def _sw_inputs(st, seed=4):
    ncol, nlay = st["play"].shape
    rng = np.random.default_rng(seed)
    for k in ("asdir", "asdif", "aldir", "aldif"):
        st[k] = rng.uniform(0.05, 0.6, ncol)
    st["coszen"] = rng.uniform(0.1, 1.0, ncol)
    return st


def test_contexts_of_a_device_agree_on_their_tables(ctx):
    st = _sw_inputs(make_state(ProfileSpec(ncol=24, nlay=38, seed=12, cloud_prob=0.6)))
    tauc = pyoracle.cldprop_columns(st)
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=2)
    ctx.sw_ini(1004.0)
    lw0 = ctx.rrtmg_lw(st, mc)
    sw0 = ctx.rrtmg_sw(st, None, icld=0, iaer=0)

    with pytest.raises(R.RrtmgLwError) as ei:
        R.Context(cpdair=1005.0)
    assert ei.value.code == GB_LW_E_TABLES

    c2 = R.Context(cpdair=1004.0)
    try:
        lw2 = c2.rrtmg_lw(st, mc)
        for k in lw0:
            if isinstance(lw0[k], np.ndarray):
                assert np.array_equal(lw2[k], lw0[k]), k
        c2.sw_ini(1004.0)
        sw2 = c2.rrtmg_sw(st, None, icld=0, iaer=0)
        with pytest.raises(R.RrtmgLwError) as ei:
            c2.sw_ini(1005.0)
        assert ei.value.code == GB_LW_E_TABLES
        with pytest.raises(R.RrtmgLwError):  # the refused load leaves c2 without shortwave tables
            c2.rrtmg_sw(st, None, icld=0, iaer=0)
    finally:
        c2.close()
    for k in ("swuflx", "swdflx", "swhr"):
        assert np.array_equal(sw2[k], sw0[k]), k
    # the live context is untouched by the refused ones
    lw1 = ctx.rrtmg_lw(st, mc)
    sw1 = ctx.rrtmg_sw(st, None, icld=0, iaer=0)
    for k in ("uflx", "dflx", "hr"):
        assert np.array_equal(lw1[k], lw0[k]), k
    for k in ("swuflx", "swdflx", "swhr"):
        assert np.array_equal(sw1[k], sw0[k]), k
