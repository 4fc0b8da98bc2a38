"""Generate the golden fixtures under tests/golden/ from the CPU oracle.

The reference ships no test vectors for this path, so these fixtures record
the oracle's own FP64 results on seeded inputs: they pin the oracle across
machines (x86 build container vs Arm GPU host) and give the GPU tests a
reference that needs no rebuild of the oracle.  Regenerate with
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle  # noqa: E402
from brams_gb300.profiles import ProfileSpec, make_state  # noqa: E402


def case(name, ncol, nlay, seed, ptop=10.0, t_noise=2.0, h2o_sigma=0.3):
    st = make_state(ProfileSpec(ncol=ncol, nlay=nlay, seed=seed, ptop=ptop, t_noise=t_noise, h2o_sigma=h2o_sigma))
    tauc = pyoracle.cldprop_columns(st)
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=1)
    out = pyoracle.rrtmg_lw(st, mc)
    arrs = {f"in_{k}": v for k, v in st.items()}
    arrs["in_tauc"] = tauc
    arrs.update({f"mc_{k}": v for k, v in mc.items()})
    arrs.update({f"out_{k}": v for k, v in out.items() if isinstance(v, np.ndarray)})
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrs)


def sw_case(name, ncol, nlay, seed, permuteseed=5):
    """The shortwave chain as BRAMS calls it: band cloud optics, the McICA
    generator (mcica_subcol_sw), then rrtmg_sw with McICA clouds (icld 3),
    aerosols (iaer 10), ice option 3, liquid option 1."""
    st = make_state(ProfileSpec(ncol=ncol, nlay=nlay, seed=seed, t_noise=3.0, h2o_sigma=0.4, cloud_prob=0.7))
    rng = np.random.default_rng(seed)
    for k in ("asdir", "asdif", "aldir", "aldif"):
        st[k] = rng.uniform(0.05, 0.6, ncol)
    st["coszen"] = rng.uniform(0.05, 1.0, ncol)
    st["coszen"][:2] = [1.0, -0.2]  # overhead sun and a night column
    # aerosol and band optics are float32 values (stored as such, exactly)
    f32 = lambda a: np.asfortranarray(a.astype(np.float32).astype(np.float64))  # noqa: E731
    st["tauaer_sw"] = f32(rng.uniform(0.0, 0.05, (ncol, nlay, 14)))
    st["ssaaer_sw"] = f32(rng.uniform(0.8, 0.99, (ncol, nlay, 14)))
    st["asmaer_sw"] = f32(rng.uniform(0.5, 0.8, (ncol, nlay, 14)))
    for k in ("rei", "rel"):
        st[k] = np.asfortranarray(np.clip(st[k], 6.0, 50.0))
    band = {"tauc": f32(rng.uniform(0.1, 10.0, (14, ncol, nlay))),
            "ssac": f32(rng.uniform(0.8, 1.0, (14, ncol, nlay))),
            "asmc": f32(rng.uniform(0.6, 0.9, (14, ncol, nlay))),
            "fsfc": f32(rng.uniform(0.0, 0.5, (14, ncol, nlay)))}
    mc = pyoracle.mcica_subcol_sw(st, band, 3, permuteseed)
    out = pyoracle.rrtmg_sw(st, mc, icld=3, iaer=10)
    arrs = {f"in_{k}": (v.astype(np.float32) if k.endswith("aer_sw") else v) for k, v in st.items()}
    arrs.update({f"band_{k}": v.astype(np.float32) for k, v in band.items()})
    # the generator's draws, as the cloudy/clear mask of the sub-columns (the
    # other McICA arrays follow from it, the band optics and the layer state)
    arrs["mc_cldfmcl"] = mc["cldfmcl"].astype(np.uint8)
    arrs.update({f"out_{k}": v for k, v in out.items() if isinstance(v, np.ndarray)})
    arrs["permuteseed"] = np.array(permuteseed)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrs)


def nomcica_case(name, ncol, nlay, seed):
    """The non-McICA driver (rrtmg_lw_rad.nomcica.f90) on layer clouds: the
    first columns carry designed fraction profiles (growing, shrinking and
    equal neighbours, blocks at the surface and the top, overcast layers,
    fractions between cldprop's 1e-20 and the transfer's 1e-6 tests); the
    outputs of random (icld 1) and maximum/random (icld 2) overlap."""
    st = make_state(ProfileSpec(ncol=ncol, nlay=nlay, seed=seed, t_noise=3.0, h2o_sigma=0.4, cloud_prob=0.6))
    cf = st["cldfrac"].copy()
    designed = [(5, [0.3, 0.6, 0.45, 0.7, 0.7, 0.2]), (nlay - 2, [0.8, 0.5]), (0, [0.4, 0.6, 0.6, 0.3]),
                (8, [5e-7, 0.3, 5e-7, 0.0, 0.6]), (3, [1.0, 1.0, 0.5, 1.0])]
    for c, (l0, prof) in enumerate(designed):
        cf[c] = 0.0
        cf[c, l0:l0 + len(prof)] = prof
    rng = np.random.default_rng(seed)
    cloudy = cf > 0
    st["cldfrac"] = np.asfortranarray(cf)
    st["clwp"] = np.asfortranarray(np.where(cloudy & (st["tlay"] > 240.0), rng.uniform(5.0, 80.0, cf.shape), 0.0))
    st["ciwp"] = np.asfortranarray(np.where(cloudy & (st["tlay"] < 268.0), rng.uniform(2.0, 40.0, cf.shape), 0.0))
    st["rel"] = np.asfortranarray(rng.uniform(4.0, 20.0, cf.shape))
    st["rei"] = np.asfortranarray(rng.uniform(20.0, 80.0, cf.shape))
    st["tauaer"] = np.asfortranarray(rng.uniform(0.0, 0.02, st["tauaer"].shape))
    arrs = {f"in_{k}": v for k, v in st.items()}
    for icld in (1, 2):
        out = pyoracle.rrtmg_lw_nomcica(st, icld)
        arrs.update({f"out{icld}_{k}": v for k, v in out.items() if isinstance(v, np.ndarray)})
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrs)


def main():
    nomcica_case("lw_nomcica_10x38", 10, 38, seed=20240603)
    sw_case("sw_8x45", 8, 45, seed=20240602)
    case("lw_16x38", 16, 38, seed=20240601)
    case("lw_8x60_top5hpa", 8, 60, seed=77, ptop=5.0, t_noise=4.0, h2o_sigma=0.5)
    seeds = np.array([1, 5489, 12345, 2**31 - 1], dtype=np.int64)
    ints = np.stack([pyoracle.mt_draws(int(s), 700)[0] for s in seeds])
    np.savez_compressed(os.path.join(HERE, "mt19937_draws.npz"), seeds=seeds, ints=ints)


if __name__ == "__main__":
    main()
