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


def test_header_is_c_and_every_declared_function_links(tmp_path):
    """include/gb_rrtmg_lw.h is plain C (C89 and C99, pedantic) and C++, and a
    C program that takes the address of every declared function links
    against the library (C linkage, the header's names)."""
    import shutil
    import subprocess

    from brams_gb300.build import build

    gcc, gxx = shutil.which("gcc"), shutil.which("g++")
    if not gcc or not gxx:
        pytest.skip("no host C compiler")
    lib = build()
    inc = os.path.join(ROOT, "include")
    hdr = os.path.join(inc, "gb_rrtmg_lw.h")
    for cmd in ([gcc, "-std=c89", "-pedantic", "-Wall", "-Werror", "-fsyntax-only", "-x", "c", hdr],
                [gcc, "-std=c99", "-pedantic", "-Wall", "-Werror", "-fsyntax-only", "-x", "c", hdr],
                [gxx, "-std=c++11", "-pedantic", "-Wall", "-Werror", "-fsyntax-only", "-x", "c++", hdr]):
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, (cmd[1], r.stderr)
    names = _declared()
    src = tmp_path / "abi.c"
    src.write_text('#include "gb_rrtmg_lw.h"\n#include <stdio.h>\nint main(void) {\n  void (*fns[])(void) = {\n'
                   + ",\n".join(f"    (void (*)(void)){n}" for n in names)
                   + '\n  };\n  printf("%d\\n", (int)(sizeof fns / sizeof fns[0]));\n  return 0;\n}\n')
    r = subprocess.run([gcc, "-std=c99", "-pedantic", "-Wall", "-Werror", "-I", inc, str(src), "-L",
                        os.path.dirname(lib), "-lgb_rrtmg_lw", "-Wl,--allow-shlib-undefined", "-o",
                        str(tmp_path / "abi")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_integration_guide_interfaces_match_the_header():
    """Every Fortran bind(C) interface INTEGRATION.md shows a maintainer has
    the argument list (names, order) of the header's prototype."""
    guide = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    hdr = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "gb_rrtmg_lw.h")).read(), flags=re.S)
    protos = {}
    for m in re.finditer(r"\b(?:int|size_t)\s+(gb_\w+)\s*\((.*?)\);", hdr, flags=re.S):
        params = [q.strip() for q in m.group(2).split(",") if q.strip() and q.strip() != "void"]
        protos[m.group(1)] = [re.findall(r"(\w+)\s*$", q)[0].lower() for q in params]
    found = 0
    for m in re.finditer(r"function\s+(gb_\w+)\s*\((.*?)\)\s*&?\s*bind\(C(?:,\s*name=\"(\w+)\")?\)", guide,
                         flags=re.S):
        name, args, cname = m.group(1), m.group(2), m.group(3) or m.group(1)  # bind(C) alone: the Fortran name
        assert name == cname and name in protos, name
        fargs = [a.strip().lower() for a in args.replace("&", "").split(",") if a.strip()]
        assert fargs == protos[name], (name, fargs, protos[name])
        found += 1
    assert found >= 15


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


# --------------------------------------------------------------------------- library shard plan
SHAPES = [(37, 45), (20, 38), (13, 60), (0, 45), (50, 45)]


def test_library_shard_plan_balances_layers():
    """gb_rrtmg_lw_shard_plan gives each rank a contiguous run of the grids'
    columns laid end to end, balanced by layers, covering every column once."""
    from brams_gb300.build import build
    from brams_gb300.shard import balanced_ranges, shard_plan

    build()
    work = np.concatenate([[nl] * nc for nc, nl in SHAPES])
    starts = np.cumsum([0] + [nc for nc, _ in SHAPES])
    for world in (1, 2, 3, 4, 7, 200):
        seen = np.zeros(work.size, dtype=int)
        ref = balanced_ranges(work, world)
        for r in range(world):
            plan = shard_plan(SHAPES, world, r)
            a, b = ref[r]
            for s, (nc, _), (c0, c1) in zip(starts, SHAPES, plan):
                assert 0 <= c0 <= c1 <= nc
                lo = min(max(a, s), s + nc)
                assert (c0, c1) == (lo - s, max(min(b, s + nc), lo) - s)
                seen[s + c0:s + c1] += 1
        assert (seen == 1).all()
        loads = [sum(nl * (c1 - c0) for (nc, nl), (c0, c1) in zip(SHAPES, shard_plan(SHAPES, world, r)))
                 for r in range(world)]
        assert max(loads) - min(loads) <= 2 * 60  # each boundary is within one column of its target


def test_library_shard_plan_rejects_bad_arguments():
    from brams_gb300.rrtmg_lw import RrtmgLwError
    from brams_gb300.shard import shard_plan

    for world, rank in ((0, 0), (2, 2), (2, -1)):
        with pytest.raises(RrtmgLwError):
            shard_plan(SHAPES, world, rank)
    with pytest.raises(RrtmgLwError):
        shard_plan([(4, 0)], 2, 0)
    assert shard_plan([], 3, 1) == []


def _grid_arrays(ncol, nlay, seed):
    """Host arrays of one grid (Fortran layouts), fused-cloud mode."""
    import pyoracle
    from brams_gb300.profiles import ProfileSpec, make_state

    st = make_state(ProfileSpec(ncol=ncol, nlay=nlay, seed=seed, t_noise=4.0, h2o_sigma=0.5, cloud_prob=0.6))
    st["tauc"] = pyoracle.cldprop_columns(st)
    st["tauaer"] = np.asfortranarray(np.random.default_rng(seed).uniform(0.0, 0.02, st["tauaer"].shape))
    out = {k: np.zeros((ncol, nlay + 1), order="F") for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt")}
    out["hr"] = np.zeros((ncol, nlay), order="F")
    out["hrc"] = np.zeros((ncol, nlay), order="F")
    return st, out


def _view(base, ptr, shape_fn):
    """The slice a descriptor pointer addresses, as a view of `base` (a
    Fortran-ordered array): element offset from the base pointer, then the
    base's strides with the column extent of the slice."""
    off = (ptr - base.ctypes.data) // base.itemsize
    assert (ptr - base.ctypes.data) % base.itemsize == 0 and off >= 0
    flat = base.ravel(order="K")
    shape = shape_fn(base.shape)
    v = np.lib.stride_tricks.as_strided(flat[off:], shape=shape, strides=base.strides)
    assert v.size == 0 or off + sum((n - 1) * s // base.itemsize for n, s in zip(shape, base.strides)) < flat.size
    return v


def _solve_slices(grids, arrays, slices):
    """The oracle on the columns each descriptor slice addresses, in place."""
    import pyoracle

    from brams_gb300.rrtmg_lw import _GRID_PTRS

    for gi, d in slices:
        st, out = arrays[gi]
        n = d.ncol

        def col(shape, n=n):
            return (n,) + shape[1:]

        sub = {}
        for k in _GRID_PTRS:
            src = st.get({"reicmcl": "rei", "relqmcl": "rel"}.get(k, k))
            if k in ("cldfmcl", "taucmcl", "ciwpmcl", "clwpmcl", "d_col_status", "sur_tau", "sur_frac", "sur_flag"):
                continue
            if src is None and k in out:
                continue
            if k == "tauc":
                sub[k] = np.asfortranarray(_view(src, getattr(d, k), lambda s: (16, n, s[2])))
            elif k in st or k in ("reicmcl", "relqmcl"):
                sub[k] = np.asfortranarray(_view(src, getattr(d, k), col))
        for k in ("rei", "rel"):
            sub[k] = sub.pop({"rei": "reicmcl", "rel": "relqmcl"}[k])
        mc = pyoracle.mcica_per_column(sub, sub["tauc"], icld=3, base_seed=d.seed0)
        res = pyoracle.rrtmg_lw(sub, mc)
        for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt", "hr", "hrc"):
            _view(out[k], getattr(d, k), col)[...] = res[k]


def _make_batch():
    from brams_gb300 import rrtmg_lw as R

    arrays = [_grid_arrays(nc, nl, 40 + i) for i, (nc, nl) in enumerate(SHAPES[:3])]
    grids = []
    for i, (st, out) in enumerate(arrays):
        a = {**st, **out}
        grids.append(R.grid_desc(st["play"].shape[0], st["play"].shape[1], a, cloud_mode=R.CLOUD_FUSED,
                                 seed0=1000 * (i + 1)))
    return arrays, grids


def _plan_rank_main(rank, world, port, q):
    import sys

    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from brams_gb300.shard import shard_grids

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    arrays, grids = _make_batch()
    mine = shard_grids(grids, world, rank)
    _solve_slices(grids, arrays, mine)
    part = [(gi, d.ncol, {k: v[int((getattr(d, k) - v.ctypes.data) // 8):][:d.ncol].copy()
                          for k, v in arrays[gi][1].items()}) for gi, d in mine]
    gathered = [None] * world
    dist.all_gather_object(gathered, part)
    if rank == 0:
        full_arrays, full_grids = _make_batch()
        _solve_slices(full_grids, full_arrays, list(enumerate(full_grids)))
        covered = [0] * len(full_grids)
        ok = True
        for r_part in gathered:
            ok &= len(r_part) > 0
            for gi, n, outs in r_part:
                c0 = covered[gi]
                for k, v in outs.items():
                    ok &= np.array_equal(v, full_arrays[gi][1][k][c0:c0 + n])
                covered[gi] += n
        ok &= covered == [g.ncol for g in full_grids]
        q.put(bool(ok))
    dist.destroy_process_group()


def test_two_rank_library_shards_match_single_process():
    """Two gloo ranks each take their slices from the library's plan and
    descriptor slicing, solve them (oracle in place of the device), and the
    gathered outputs equal one process solving the whole batch: the slices'
    pointer offsets address the right columns of every array layout and the
    McICA seeds advance with the slice."""
    import multiprocessing as mp
    import socket

    from brams_gb300.build import build

    build()
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_plan_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(180)
    assert all(p.exitcode == 0 for p in ps)
    assert q.get(timeout=5) is True
