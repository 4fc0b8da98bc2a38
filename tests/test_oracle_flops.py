"""The operation-counting copy of the oracle (oracle/flop_count.h): same
outputs as the oracle, and per-phase counts that add up and scale with the
work of each phase."""
import numpy as np

import pyoracle
from brams_gb300.profiles import ProfileSpec, make_state


def _case(ncol, nlay, seed):
    st = make_state(ProfileSpec(ncol=ncol, nlay=nlay, seed=seed, t_noise=4.0, h2o_sigma=0.5))
    tauc = pyoracle.cldprop_columns(st)
    return st, pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=1)


def test_counting_copy_gives_the_oracles_outputs():
    st, mc = _case(8, 38, 3)
    r = pyoracle.flops_per_column(st, mc)
    ref = pyoracle.rrtmg_lw(st, mc)
    for k in ("uflx", "dflx", "hr", "uflxc", "dflxc", "hrc", "duflx_dt", "duflxc_dt"):
        assert np.array_equal(r["outputs"][k], ref[k]), k


def test_phase_counts():
    st, mc = _case(8, 45, 4)
    r = pyoracle.flops_per_column(st, mc)
    phases = ("inatm", "cldprmc", "setcoef", "taumol", "rtrnmc")
    assert all(r[p] > 0 for p in phases)
    assert abs(sum(r[p] for p in phases) - r["total"]) < 1e-9 * r["total"]
    # taumol and rtrnmc work per (layer, g-point) cell dominates
    assert r["taumol"] + r["rtrnmc"] > 0.9 * r["total"]
    assert 10 < r["taumol"] / (45 * 140) < 60 and 20 < r["rtrnmc"] / (45 * 140) < 80
    # twice the layers, about twice the work
    st2, mc2 = _case(8, 90, 4)
    r2 = pyoracle.flops_per_column(st2, mc2)
    assert 1.6 < r2["rtrnmc"] / r["rtrnmc"] < 2.4
