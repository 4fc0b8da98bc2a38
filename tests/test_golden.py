"""Oracle against the committed golden fixtures (CPU) and the CUDA library
against the same fixtures (GPU): two longwave cases (McICA sub-columns and
outputs) and the shortwave chain (the generator's sub-column mask from band
cloud optics, then rrtmg_sw with McICA clouds and aerosols)."""
import os

import numpy as np
import pytest

import pyoracle

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["lw_16x38", "lw_8x60_top5hpa"]
OUTS = ["uflx", "dflx", "uflxc", "dflxc", "hr", "hrc", "duflx_dt", "duflxc_dt"]


def _load(name):
    z = np.load(os.path.join(G, name + ".npz"))
    st = {k[3:]: np.asfortranarray(z[k]) for k in z.files if k.startswith("in_")}
    mc = {k[3:]: np.asfortranarray(z[k]) for k in z.files if k.startswith("mc_")}
    out = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return st, mc, out


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_golden(name):
    st, mc, ref = _load(name)
    mc2 = pyoracle.mcica_per_column(st, st.pop("tauc"), icld=3, base_seed=1)
    for k in mc:
        assert np.array_equal(mc2[k], mc[k]), k  # McICA draws are integer-exact on every machine
    out = pyoracle.rrtmg_lw(st, mc)
    for k in OUTS:
        # libm exp/log/pow may differ in the last bit between machines
        assert np.allclose(out[k], ref[k], rtol=1e-10, atol=1e-10), k


def test_mt_golden():
    z = np.load(os.path.join(G, "mt19937_draws.npz"))
    for s, ints in zip(z["seeds"], z["ints"]):
        assert np.array_equal(pyoracle.mt_draws(int(s), ints.size)[0], ints)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_golden(ctx, name):
    st, mc, ref = _load(name)
    tauc = st.pop("tauc")
    gmc = ctx.mcica_subcol_lw(st, tauc, icld=3, permuteseed=1, seed_per_column=True)
    for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl"):
        assert np.array_equal(gmc[k], mc[k]), k
    out = ctx.rrtmg_lw(st, mc)
    for k in ("uflx", "dflx", "uflxc", "dflxc"):
        assert np.abs(out[k] - ref[k]).max() <= 0.05, k
    for k in ("hr", "hrc"):
        assert np.abs(out[k] - ref[k]).max() <= 0.01, k


SW_OUTS = ["swuflx", "swdflx", "swuflxc", "swdflxc", "swhr", "swhrc"]


def _load_sw(name="sw_8x45"):
    z = np.load(os.path.join(G, name + ".npz"))
    st = {k[3:]: np.asfortranarray(z[k].astype(np.float64)) for k in z.files if k.startswith("in_")}
    band = {k[5:]: np.asfortranarray(z[k].astype(np.float64)) for k in z.files if k.startswith("band_")}
    out = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return st, band, z["mc_cldfmcl"].astype(np.float64), int(z["permuteseed"]), out


def test_oracle_reproduces_sw_golden():
    st, band, cldf, seed, ref = _load_sw()
    mc = pyoracle.mcica_subcol_sw(st, band, 3, seed)
    assert np.array_equal(mc["cldfmcl"], cldf)
    assert 0.05 < cldf.mean() < 0.9
    out = pyoracle.rrtmg_sw(st, mc, icld=3, iaer=10)
    for k in SW_OUTS:
        assert np.allclose(out[k], ref[k], rtol=1e-10, atol=1e-10), k
    assert ref["swdflx"][1].max() < 1e-6    # the night column (cos zenith floored at 1e-10)
    assert ref["swdflx"][0, -1] > 1000.0    # overhead sun: incoming flux at the top


@pytest.mark.gpu
@pytest.mark.parametrize("bits", [64, 32])
def test_gpu_matches_sw_golden(ctx, bits):
    st, band, cldf, seed, ref = _load_sw()
    ctx.sw_ini(1004.0)
    mc = ctx.mcica_subcol_sw(st, band, 3, seed)
    assert np.array_equal(mc["cldfmcl"], cldf)
    ctx.sw_set_precision(bits)
    try:
        out = ctx.rrtmg_sw(st, mc, icld=3, iaer=10)
    finally:
        ctx.sw_set_precision(32)
    flux_tol, hr_tol = (1e-6, 1e-8) if bits == 64 else (0.05, 0.01)
    for k in ("swuflx", "swdflx", "swuflxc", "swdflxc"):
        assert np.abs(out[k] - ref[k]).max() <= flux_tol, k
    for k in ("swhr", "swhrc"):
        assert np.abs(out[k] - ref[k]).max() <= hr_tol, k


def _load_nomcica(name="lw_nomcica_10x38"):
    z = np.load(os.path.join(G, name + ".npz"))
    st = {k[3:]: np.asfortranarray(z[k]) for k in z.files if k.startswith("in_")}
    outs = {icld: {k[5:]: z[k] for k in z.files if k.startswith(f"out{icld}_")} for icld in (1, 2)}
    return st, outs


@pytest.mark.parametrize("icld", [1, 2])
def test_oracle_reproduces_nomcica_golden(icld):
    st, outs = _load_nomcica()
    out = pyoracle.rrtmg_lw_nomcica(st, icld)
    for k in OUTS:
        assert np.allclose(out[k], outs[icld][k], rtol=1e-10, atol=1e-10), k
    assert np.abs(out["dflx"] - out["dflxc"]).max() > 1.0  # the clouds are seen


@pytest.mark.gpu
@pytest.mark.parametrize("icld", [1, 2])
def test_gpu_matches_nomcica_golden(ctx, icld):
    st, outs = _load_nomcica()
    out = ctx.rrtmg_lw_nomcica(st, icld)
    ref = outs[icld]
    for k in ("uflx", "dflx", "uflxc", "dflxc"):
        assert np.abs(out[k] - ref[k]).max() <= 0.05, k
    for k in ("hr", "hrc"):
        assert np.abs(out[k] - ref[k]).max() <= 0.01, k
    for k in ("duflx_dt", "duflxc_dt"):
        assert np.abs(out[k] - ref[k]).max() <= 1e-3, k
