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


def main():
    case("lw_16x38", 16, 38, seed=20240601)
    case("lw_8x60_top5hpa", 8, 60, seed=77, ptop=5.0, t_noise=4.0, h2o_sigma=0.5)
    seeds = np.array([1, 5489, 12345, 2**31 - 1], dtype=np.int64)
    ints = np.stack([pyoracle.mt_draws(int(s), 700)[0] for s in seeds])
    np.savez_compressed(os.path.join(HERE, "mt19937_draws.npz"), seeds=seeds, ints=ints)


if __name__ == "__main__":
    main()
