"""Allocation-free McICA entry point (gb_mcica_subcol_lw_noalloc) through the C ABI.

Some callers cannot allocate device memory while their model runs (device
memory owned by another runtime or pool, or steps that must not take the
synchronisation cudaMalloc/cudaFree can cause).  This entry point keeps its
draw scratch in a fixed array inside the library.  The test checks, on two
calls in a row, that its output equals the allocating entry point's
(bit for bit, as for every McICA test) and that device free memory does not
move across the calls.  The file name sorts last so a -x run has already run
every other test if this one fails.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OUTS = ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl")
INS = ("play", "cldfrac", "ciwp", "clwp", "rei", "rel", "tauc", "alpha")


def _inputs(ncol, nlay, seed):
    import torch

    import pyoracle
    from brams_gb300.profiles import ProfileSpec, make_state

    st = make_state(ProfileSpec(ncol=ncol, nlay=nlay, seed=seed, t_noise=4.0, h2o_sigma=0.5))
    tauc = pyoracle.cldprop_columns(st)
    dev = torch.device("cuda", 0)

    def dv(a):
        return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).to(dev)

    d = {k: dv(st[k]) for k in ("play", "cldfrac", "ciwp", "clwp", "rei", "rel")}
    d["tauc"] = dv(tauc)
    alpha = np.exp(-np.linspace(0.1, 2.0, nlay))[None, :] * np.ones((ncol, 1))
    d["alpha"] = dv(alpha)
    return d


def _outputs(ncol, nlay):
    import torch

    dev = torch.device("cuda", 0)
    o = {k: torch.full((nlay, ncol, 140), -1.0, dtype=torch.float64, device=dev) for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl")}
    o["reicmcl"] = torch.full((nlay, ncol), -1.0, dtype=torch.float64, device=dev)
    o["relqmcl"] = torch.full((nlay, ncol), -1.0, dtype=torch.float64, device=dev)
    return o


def test_noalloc_matches_allocating_entry_point():
    import torch

    from brams_gb300.build import build
    from brams_gb300.rrtmg_lw import Context, load_library

    build()
    L = load_library()
    ctx = Context()
    stream = torch.cuda.current_stream().cuda_stream
    ncol, nlay = 3000, 45
    calls = [  # (icld, permuteseed, irng, seed_per_column): two calls in a row, then other modes
        (3, 11, 1, 1),
        (3, 12345, 1, 0),
        (2, 7, 0, 1),
        (4, 5, 1, 1),  # exponential overlap: two draws per cell and the overlap parameter
    ]
    d = _inputs(ncol, nlay, seed=5)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    for n, (icld, seed, irng, percol) in enumerate(calls):
        ncall = ncol if icld == 3 else (400 if icld == 2 else 200)  # icld 2/4 need 140*nlay (x2) draws per column
        got = _outputs(ncol, nlay)
        ref = _outputs(ncol, nlay)
        ir = C.c_int(irng)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = L.gb_mcica_subcol_lw_noalloc(
            C.c_void_p(stream), ncall, nlay, icld, seed, C.byref(ir),
            *[C.c_void_p(d[k].data_ptr()) for k in INS],
            *[C.c_void_p(got[k].data_ptr()) for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl")],
            ncol, percol, C.c_void_p(status.data_ptr()))
        assert rc == 0, L.gb_rrtmg_lw_strerror(rc)
        torch.cuda.synchronize()
        if n > 0:  # the first call on the device may load the library's module (set-up)
            assert torch.cuda.mem_get_info()[0] == free_before  # nothing allocated by the call
        assert int(status.item()) == 0
        ctx.mcica_subcol_lw_device(ncall, nlay, {**d, **ref}, icld=icld, permuteseed=seed, irng=irng,
                                   seed_per_column=bool(percol), stream=stream, ld=ncol)
        torch.cuda.synchronize()
        for k in OUTS:
            a, b = got[k][:, :ncall], ref[k][:, :ncall]
            assert torch.equal(a, b), (n, k)
        assert float(got["cldfmcl"][:, :ncall].sum()) > 0  # clouds were generated
    ctx.close()


def test_noalloc_rejects_calls_beyond_its_scratch():
    import torch

    from brams_gb300.rrtmg_lw import load_library

    L = load_library()
    ir = C.c_int(1)
    big = 4 * 1024 * 1024 // 140 + 1  # icld 3 needs 140 draws per column
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    rc = L.gb_mcica_subcol_lw_noalloc(None, big, 10, 3, 1, C.byref(ir), *([p] * 8), *([p] * 6), big, 1, None)
    assert rc == -5
    assert b"scratch" in L.gb_rrtmg_lw_strerror(rc)


def test_noalloc_reports_the_kiss_seeding_stop():
    """KISS seeding needs the bottom layers' pressures in decreasing order
    (the reference stops otherwise): the call reports status 8 and gives the
    same sub-columns on a repeated call (zero draws, not stale ones)."""
    import torch

    from brams_gb300.rrtmg_lw import load_library

    L = load_library()
    stream = torch.cuda.current_stream().cuda_stream
    ncol, nlay = 64, 20
    good = _inputs(ncol, nlay, seed=9)
    bad = _inputs(ncol, nlay, seed=9)
    bad["play"][[0, 1], 3] = bad["play"][[1, 0], 3]  # column 3: pmid(1) < pmid(2)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    OUT = ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl", "relqmcl", "taucmcl")

    def call(d, seed):
        got = _outputs(ncol, nlay)
        ir = C.c_int(0)
        rc = L.gb_mcica_subcol_lw_noalloc(
            C.c_void_p(stream), ncol, nlay, 2, seed, C.byref(ir), *[C.c_void_p(d[k].data_ptr()) for k in INS],
            *[C.c_void_p(got[k].data_ptr()) for k in OUT], ncol, 1, C.c_void_p(status.data_ptr()))
        assert rc == 0
        torch.cuda.synchronize()
        return got, int(status.item())

    res = []
    for seed in (100, 200):  # a clean call with other draws, then the failing one
        _, st = call(good, seed)
        assert st == 0
        got, st = call(bad, 1)
        assert st == 8  # GB_LW_E_KISS_PMID
        res.append(got["cldfmcl"][:, 3].clone())
    assert torch.equal(res[0], res[1])
