"""The non-McICA driver on the GPU (gb_rrtmg_lw_nomcica): cldprop on band-level
clouds, then random overlap (rtrn, icld 1) or maximum/random overlap (rtrnmr,
icld 2 and 3; icld 0 clear), against the FP64 oracle's restatement of
rrtmg_lw_rad.nomcica.f90.

The designed columns put cloud-fraction profiles through every branch of
rtrnmr's overlap-factor set-up (rrtmg_lw_rtrnmr.f90:345-514): growing,
shrinking and equal neighbours, blocks that start at the surface and end at
the model top, overcast blocks, and fractions between cldprop's 1e-20 and
the transfer's 1e-6 cloud tests.  Every cloud option of cldprop runs, which
also gives all three cloud-band counts (1, 5 and 16).

Tolerances: fluxes within 0.05 W m-2, heating rates within 0.01 K/day,
surface-temperature derivatives within 1e-3 W m-2 K-1.
"""
import numpy as np
import pytest

import pyoracle
from brams_gb300.profiles import ProfileSpec, make_state

FLUX_TOL, HR_TOL, DER_TOL = 0.05, 0.01, 1e-3
PROFILES = [
    # (first layer, fractions upward)
    (5, [0.3, 0.6, 0.45, 0.7, 0.7, 0.2]),
    (None, [0.8, 0.5]),               # the two top layers
    (0, [0.4, 0.6, 0.6, 0.3]),        # from the surface up
    (8, [5e-7, 0.3, 5e-7, 0.0, 0.6]),  # fractions cldprop counts and the transfer does not
    (3, [1.0, 1.0, 0.5, 1.0]),
    (12, [0.2, 0.5, 0.9, 0.4, 0.1]),
    (20, [0.6, 0.3, 0.3, 0.8]),
    (2, [0.5, 0.25, 0.75, 0.25, 0.5]),
]


def overlap_state(ncol=24, nlay=38, seed=515):
    """Designed fraction profiles in the first columns, the generator's own
    (probability 0.6) in the rest; liquid and ice water where cloudy."""
    st = make_state(ProfileSpec(ncol=ncol, nlay=nlay, seed=seed, t_noise=3.0, h2o_sigma=0.4, cloud_prob=0.6))
    cf = st["cldfrac"].copy()
    for c, (l0, prof) in enumerate(PROFILES):
        cf[c] = 0.0
        start = nlay - len(prof) if l0 is None else l0
        cf[c, start:start + len(prof)] = prof
    rng = np.random.default_rng(seed)
    cloudy = cf > 0
    st["cldfrac"] = np.asfortranarray(cf)
    st["clwp"] = np.asfortranarray(np.where(cloudy & (st["tlay"] > 240.0), rng.uniform(5.0, 80.0, cf.shape), 0.0))
    st["ciwp"] = np.asfortranarray(np.where(cloudy & (st["tlay"] < 268.0), rng.uniform(2.0, 40.0, cf.shape), 0.0))
    st["rel"] = np.asfortranarray(rng.uniform(4.0, 20.0, cf.shape))
    st["rei"] = np.asfortranarray(rng.uniform(20.0, 80.0, cf.shape))
    st["tauaer"] = np.asfortranarray(rng.uniform(0.0, 0.02, st["tauaer"].shape))
    st["tauc_band"] = np.asfortranarray(np.where(cloudy.T[None], rng.uniform(0.1, 8.0, (16, nlay, ncol)), 0.0)
                                        .transpose(0, 2, 1))
    return st


def _branches(cf):
    """The branches of rtrnmr's overlap set-up a column's fractions take
    (upward and downward loops), as (direction, case) labels."""
    nl = len(cf)
    CF = lambda lev: cf[lev - 1] if 1 <= lev <= nl else 0.0  # noqa: E731
    cloudy = [None] + [CF(lev) >= 1e-6 for lev in range(1, nl + 1)]
    seen = set()
    st = 1
    for lev in range(1, nl + 1):
        if not cloudy[lev]:
            st = 1
            continue
        c0, cp, cm = CF(lev), CF(lev + 1), CF(lev - 1)
        if lev == nl:
            seen.add(("up", "top"))
        elif cp >= c0:
            seen.add(("up", "grow-first") if st else ("up", "grow-above" if cp > max(c0, cm) else
                                                      "grow-below" if cp < max(c0, cm) else "grow-equal"))
        else:
            seen.add(("up", "shrink-first") if st else ("up", "shrink-below" if cp <= min(c0, cm) else "shrink-within"))
        st = 0
    sd = 1
    for lev in range(nl, 0, -1):
        if not cloudy[lev]:
            sd = 1
            continue
        c0, cp, cm = CF(lev), CF(lev + 1), CF(lev - 1)
        if lev == 1:
            seen.add(("dn", "bottom"))
        elif cm >= c0:
            seen.add(("dn", "grow-first") if sd else ("dn", "grow-above" if cm > max(c0, cp) else
                                                      "grow-below" if cm < max(c0, cp) else "grow-equal"))
        else:
            seen.add(("dn", "shrink-first") if sd else ("dn", "shrink-below" if cm <= min(c0, cp) else "shrink-within"))
        sd = 0
    return seen


def test_designed_profiles_reach_every_overlap_branch():
    st = overlap_state()
    seen = set()
    for c in range(st["cldfrac"].shape[0]):
        seen |= _branches(st["cldfrac"][c])
    cases = ["grow-first", "grow-above", "grow-below", "grow-equal", "shrink-first", "shrink-below", "shrink-within"]
    want = {(d, k) for d in ("up", "dn") for k in cases} | {("up", "top"), ("dn", "bottom")}
    assert want <= seen, sorted(want - seen)
    # fractions that cldprop counts as cloud and the transfer does not
    assert ((st["cldfrac"] >= 1e-20) & (st["cldfrac"] < 1e-6)).any()


def _parity(out, ref, idrv=1):
    for k in ("uflx", "dflx", "uflxc", "dflxc"):
        assert np.abs(out[k] - ref[k]).max() <= FLUX_TOL, (k, float(np.abs(out[k] - ref[k]).max()))
    for k in ("hr", "hrc"):
        assert np.abs(out[k] - ref[k]).max() <= HR_TOL, (k, float(np.abs(out[k] - ref[k]).max()))
    if idrv == 1:
        for k in ("duflx_dt", "duflxc_dt"):
            assert np.abs(out[k] - ref[k]).max() <= DER_TOL, (k, float(np.abs(out[k] - ref[k]).max()))


@pytest.mark.gpu
@pytest.mark.parametrize("icld", [0, 1, 2, 3, 7])
def test_overlap_methods_match_oracle(ctx, icld):
    st = overlap_state()
    ref = pyoracle.rrtmg_lw_nomcica(st, icld)
    out = ctx.rrtmg_lw_nomcica(st, icld)
    assert out["icld"] == ref["icld"] == (2 if icld == 7 else icld)
    _parity(out, ref)
    if icld >= 1:
        assert np.abs(out["dflx"] - out["dflxc"]).max() > 1.0  # the clouds are seen


@pytest.mark.gpu
@pytest.mark.parametrize("flags", [(2, 0, 0), (2, 1, 0), (2, 1, 1), (2, 2, 1), (2, 3, 0), (0, 3, 1), (1, 3, 1)])
@pytest.mark.parametrize("icld", [1, 2])
def test_cloud_options_match_oracle(ctx, flags, icld):
    """inflag/iceflag/liqflag: (2,0,0) one cloud band, (2,1,0) five, the rest 16."""
    inflag, iceflag, liqflag = flags
    st = overlap_state(seed=600 + 10 * inflag + iceflag + 4 * liqflag)
    rng = np.random.default_rng(9)
    if iceflag == 0:
        st["rei"] = np.asfortranarray(rng.uniform(12.0, 120.0, st["rei"].shape))
    elif iceflag == 1:
        st["rei"] = np.asfortranarray(rng.uniform(14.0, 125.0, st["rei"].shape))
    kw = dict(inflglw=inflag, iceflglw=iceflag, liqflglw=liqflag)
    ref = pyoracle.rrtmg_lw_nomcica(st, icld, **kw)
    out = ctx.rrtmg_lw_nomcica(st, icld, **kw)
    _parity(out, ref)


@pytest.mark.gpu
def test_device_entry_matches_host_entry_and_reports_radius_stops(ctx):
    import torch

    from brams_gb300 import rrtmg_lw as R

    st = overlap_state(ncol=20, seed=77)
    st["ciwp"][4, 3] = 5.0
    st["rei"][4, :] = 200.0  # column 4: ice size beyond iceflag 3's bounds where it has ice
    assert st["cldfrac"][4, 3] >= 1e-20
    ncol, nlay = st["play"].shape
    dev = torch.device("cuda", 0)

    def dv(a):
        return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)).to(dev)

    d = {k: dv(st[k]) for k in R.STATE_ORDER + ["tauaer", "cldfrac", "ciwp", "clwp", "rei", "rel", "tauc_band"]}
    for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt"):
        d[k] = torch.zeros((nlay + 1, ncol), dtype=torch.float64, device=dev)
    d["hr"] = torch.zeros((nlay, ncol), dtype=torch.float64, device=dev)
    d["hrc"] = torch.zeros((nlay, ncol), dtype=torch.float64, device=dev)
    status = torch.full((ncol,), -1, dtype=torch.int32, device=dev)
    ctx.rrtmg_lw_nomcica_device(ncol, nlay, d, icld=2, col_status=status)
    torch.cuda.synchronize()
    s = status.cpu().numpy()
    assert s[4] == 5 and (np.delete(s, 4) == 0).all()  # GB_LW_E_DGE_BOUNDS, that column only
    assert ctx.sync_status() == 5
    ok = [c for c in range(ncol) if c != 4]
    sub = {k: (np.asfortranarray(v[:, ok]) if k == "tauc_band" else np.asfortranarray(v[ok]))
           for k, v in st.items()}
    host = ctx.rrtmg_lw_nomcica(sub, 2)
    for k in ("uflx", "dflx", "uflxc", "dflxc", "hr", "hrc", "duflx_dt", "duflxc_dt"):
        got = d[k].cpu().numpy().T[ok]
        assert np.array_equal(got, host[k]), k
