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


def test_sw_counting_copy():
    """The shortwave restatement's counting copy: the oracle's outputs, and a
    count per column that grows with the layers (cells of 112 g-points)."""
    from test_sw import sw_mcica, sw_state

    st, st2 = sw_state(ncol=6, nlay=30, seed=3, cloud_prob=0.6), sw_state(ncol=6, nlay=60, seed=3, cloud_prob=0.6)
    mc, mc2 = sw_mcica(st, seed=2), sw_mcica(st2, seed=2)
    ref = pyoracle.rrtmg_sw(st, mc, icld=3, iaer=10)
    got = pyoracle.rrtmg_sw(st, mc, icld=3, iaer=10, _count=True)
    for k in ("swuflx", "swdflx", "swhr", "swuflxc", "swdflxc", "swhrc"):
        assert np.array_equal(got[k], ref[k]), k
    f1 = pyoracle.sw_flops_per_column(st, mc, icld=3, iaer=10)
    f2 = pyoracle.sw_flops_per_column(st2, mc2, icld=3, iaer=10)
    assert 100 < f1 / (30 * 112) < 1000
    assert 1.6 < f2 / f1 < 2.4
