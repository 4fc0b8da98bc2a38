"""C ABI surface (library loads, exports every declared symbol) and the
multi-process column sharding (gloo ranks on CPU)."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "gb_rrtmg_lw.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from brams_gb300.build import build

    lib = build()
    import ctypes

    L = ctypes.CDLL(lib)
    names = _declared()
    assert len(names) >= 10
    for n in names:
        assert hasattr(L, n), n
    from brams_gb300.rrtmg_lw import EXPORTS

    assert sorted(EXPORTS) == names


def test_library_init_without_gpu_fails_cleanly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from brams_gb300.rrtmg_lw import Context, RrtmgLwError

    with pytest.raises(RrtmgLwError):
        Context()


def test_balanced_ranges():
    from brams_gb300.shard import balanced_ranges, column_ranges

    r = column_ranges(10, 3)
    assert r[0][0] == 0 and r[-1][1] == 10 and all(a[1] == b[0] for a, b in zip(r, r[1:]))
    w = np.array([45] * 100 + [38] * 60)
    rr = balanced_ranges(w, 4)
    loads = [w[a:b].sum() for a, b in rr]
    assert max(loads) - min(loads) <= 45
    assert balanced_ranges(np.ones(2), 4)[-1][1] == 2


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from brams_gb300.profiles import ProfileSpec, make_state
    from brams_gb300.shard import column_ranges

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    st = make_state(ProfileSpec(ncol=10, nlay=20, seed=17))
    tauc = pyoracle.cldprop_columns(st)
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=1)
    a, b = column_ranges(10, world)[rank]
    sub = {k: np.asfortranarray(v[a:b]) for k, v in st.items()}
    smc = {k: np.asfortranarray(v[:, a:b] if v.ndim == 3 else v[a:b]) for k, v in mc.items()}
    out = pyoracle.rrtmg_lw(sub, smc)
    gathered = [None] * world
    dist.all_gather_object(gathered, (a, b, out["uflx"], out["hr"]))
    if rank == 0:
        full = pyoracle.rrtmg_lw(st, mc)
        ok = all(np.array_equal(u, full["uflx"][a:b]) and np.array_equal(h, full["hr"][a:b]) for a, b, u, h in gathered)
        q.put(ok)
    dist.destroy_process_group()


def test_two_rank_column_shards_match_single_process():
    import multiprocessing as mp
    import socket

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
    assert all(p.exitcode == 0 for p in ps)
    assert q.get(timeout=5) is True
