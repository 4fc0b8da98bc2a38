"""Benchmark of the GB300 RRTMG_LW column solver.

Headline workload (the metric's own configuration): 2048x1024 columns x 60
layers (pressure 1000 -> 5 hPa) x 4 ensemble members = 8,388,608 columns in
all, McICA clouds generated in the kernel (icld 3, seed = base + column), FP32
transfer with FP64 heating rates.  One step solves every column once by:

  surrogate  -- the learned gas optics (brams_gb300/data/lw_mlp.gbmlp) with
                per-layer fallback to taumol: per chunk of columns the MLP
                inference kernel, then one batched launch of the column
                kernel over the four members;
  plain      -- taumol: one batched launch of the column kernel over the four
                members (no learned part).

  value        -- columns/s of the surrogate path, inputs resident in HBM
                  (~90 GB per step, far larger than the 129 MB L2: no flush)
  plain_gpu    -- columns/s of the plain path on the same inputs; speedup
  accuracy     -- heating-rate RMSE of both paths against the FP64 oracle on
                  a contiguous sample of member 0's columns
  e2e          -- the surrogate path with every step's inputs copied from
                  page-locked host memory chunk by chunk and every output read
                  back (host data: the generator tile, streamed for every chunk)
  roofline     -- the dominant kernel (the transfer kernel on the network's
                  gas optics, fused clouds) against the measured HBM copy
                  bandwidth with its algorithmic bytes, and against the
                  nominal FP32 peak with the operations the oracle's counting
                  copy counts for its phases (inatm, cldprmc, rtrnmc)
  batched      -- three nested grids (200x180x45, 150x150x45, 97x97x38) x 8
                  ensemble members with perturbed T and H2O, all in one
                  persistent launch captured in a CUDA graph (taumol, fused
                  clouds), with HBM and FP32 rooflines and an oracle check
  eval         -- the learned gas optics on 512x512x45 columns: columns/s
                  and heating-rate RMSE against the FP64 oracle, beside the
                  plain path
  nomcica      -- the non-McICA driver (cldprop, taumol, random or
                  maximum/random overlap) on 360x300x45 device arrays
  shortwave    -- RRTMG_SW (McICA generator and solver in both precisions)
                  on 360x300x45 device arrays (--sw-ncol), their error
                  against the FP64 oracle, FP32/FP64 rooflines from counted
                  operations and the oracle's throughput on the host cores
                  (--no-sw skips it, --no-cpu its oracle parts)
  plain_abi    -- the drop-in path on the 360x300x45 BRAMS-scale workload:
                  gb_rrtmg_lw_device on the reference's (140, ncol, nlay)
                  McICA arrays, its roofline against 8*(600*nlay + 25) bytes
                  per column, and gb_rrtmg_lw with page-locked host buffers
  cpu_baseline -- the FP64 oracle (C++ restatement of the reference) on the
                  host cores, on a bounded sample of the headline workload;
                  cpu_configs: the same on the 64x64x38 configuration in full
                  and on a sample of the 360x300x45 one

Inputs: a 131,072-column tile from the seeded generator (T noise N(0, 4 K),
H2O x lognormal(0, 0.5)) is replicated to the 2048x1024 grid with a fresh
T + N(0, 1 K), H2O x lognormal(0, 0.2) perturbation per replica, and each
ensemble member perturbs T and H2O again the same way.

``--impl reference`` times the CPU implementation alone (the reference's
Fortran cannot be built on this machine; its C++ restatement is timed instead).
Multi-GPU (torchrun): each rank solves its own full workload (weak scaling,
no collective on the data path); value = all ranks' columns / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "LW columns/s, surrogate vs plain GPU, at <=0.1 K/day heating-rate RMSE"
NCOL, NLAY, PTOP = 360 * 300, 45, 10.0          # drop-in block (BRAMS operational scale)
NX, NY, NMEM, NLAY5, PTOP5 = 2048, 1024, 4, 60, 5.0  # headline workload
TILE = 131072                                    # generator tile replicated over the grid
CHUNK = 65536                                    # columns per member per surrogate call
BASE_SEED = 1
SAMPLE = 2048                                    # oracle columns for the accuracy check


def abi_bytes_per_column(nlay: int) -> int:
    return 8 * (600 * nlay + 25)


# FP32 peak of a GB300 by its nominal figures (no measured FP32 peak is
# available): 152 SMs x 128 FP32 lanes x 2 operations (FMA) x 2.07 GHz
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12
FP64_PEAK_TFLOPS = 1.25  # GB300 dense FP64, nominal


def counted_flops(st: dict, mc: dict) -> dict:
    """Floating-point operations per column by phase, counted by the
    oracle's counting copy on these columns (single-threaded)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    r = pyoracle.flops_per_column(st, mc)
    r.pop("outputs")
    return r


# --------------------------------------------------------------------------- inputs
def cldprop_numpy(st: dict, tabs: dict) -> np.ndarray:
    """Band cloud optical depth as BRAMS computes it with cldprop for the McICA
    tauc argument (rrtmg_lw_cldprop.f90:50-295, inflag 2, iceflag 3, liqflag 1);
    vectorised input preparation, not part of the timed solver."""
    cf, ci, cw, re, rl = st["cldfrac"], st["ciwp"], st["clwp"], st["rei"], st["rel"]
    ncol, nlay = cf.shape
    tau = np.zeros((16, ncol, nlay), order="F")
    cloudy = (cf >= 1e-20) & ((ci + cw) >= 1e-20)
    fac = (re - 2.0) / 3.0
    idx = np.clip(fac.astype(np.int64), 1, 45)
    fint = fac - idx
    il = np.clip((rl - 1.5).astype(np.int64), 1, 57)
    fl = rl - 1.5 - il
    a3, a1 = tabs["absice3"], tabs["absliq1"]
    for b in range(16):
        ai = a3[idx - 1, b] + fint * (a3[idx, b] - a3[idx - 1, b])
        al = a1[il - 1, b] + fl * (a1[il, b] - a1[il - 1, b])
        ai = np.where(ci == 0.0, 0.0, ai)
        al = np.where(cw == 0.0, 0.0, al)
        tau[b] = np.where(cloudy, ci * ai + cw * al, 0.0)
    return tau


def make_inputs(ncol: int, nlay: int, seed: int):
    from brams_gb300.profiles import ProfileSpec, make_state
    from brams_gb300.tables_io import read_tables

    st = make_state(ProfileSpec(ncol=ncol, nlay=nlay, seed=seed, ptop=PTOP, t_noise=4.0, h2o_sigma=0.5))
    tabs = read_tables(os.path.join(ROOT, "brams_gb300", "data", "lw_ref_tables.gblw"))
    return st, cldprop_numpy(st, tabs)


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(2)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# --------------------------------------------------------------------------- CPU baseline
def cpu_baseline(st, mc, max_seconds: float = 12.0):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    try:
        pyoracle.build(tuned=True)
        tuned = True
    except Exception:
        tuned = False
    cores = os.cpu_count() or 1
    ncol = st["play"].shape[0]

    def sub(n):
        s = {k: np.asfortranarray(v[:n]) for k, v in st.items()}
        m = {k: np.asfortranarray(v[:, :n] if v.ndim == 3 else v[:n]) for k, v in mc.items()}
        return s, m

    probe = min(ncol, 64 * cores)
    s, m = sub(probe)
    t0 = time.perf_counter()
    pyoracle.rrtmg_lw(s, m, nthreads=cores, tuned=tuned)
    dt = time.perf_counter() - t0
    n = int(min(ncol, max(probe, probe * max_seconds / max(dt, 1e-6))))
    s, m = sub(n)
    t0 = time.perf_counter()
    pyoracle.rrtmg_lw(s, m, nthreads=cores, tuned=tuned)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "columns/s", "cores": cores, "kind": "port",
            "sample": f"first {n} of {ncol} columns of the 360x300x45 workload, one pass, "
                      f"{cores} threads, FP64 C++ restatement ({'-O3, Neoverse V2 tuning on aarch64' if tuned else '-O2'})"}


def reference_arm(args, rank, world):
    """--impl reference: the CPU implementation alone (FP64 C++ restatement of
    the reference, all host threads) on columns of the headline workload."""
    if rank != 0:
        return
    from brams_gb300.profiles import ProfileSpec, make_state
    from brams_gb300.tables_io import read_tables

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build(tuned=True)
    cores = os.cpu_count() or 1
    n = max(256, 256 * cores)
    st = make_state(ProfileSpec(ncol=n, nlay=NLAY5, seed=BASE_SEED, ptop=PTOP5, t_noise=4.0, h2o_sigma=0.5))
    tabs = read_tables(os.path.join(ROOT, "brams_gb300", "data", "lw_ref_tables.gblw"))
    tauc = cldprop_numpy(st, tabs)
    mc = pyoracle.mcica_per_column(st, tauc, icld=3, base_seed=BASE_SEED)
    for _ in range(args.warmup):
        pyoracle.rrtmg_lw(st, mc, nthreads=cores, tuned=True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pyoracle.rrtmg_lw(st, mc, nthreads=cores, tuned=True)
    dt = (time.perf_counter() - t0) / args.steps
    v = n / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "columns/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"rrtmg_lw on {n} columns per step of the {NX}x{NY} x {NLAY5}-layer "
                                   f"({NMEM}-member) workload", "columns_per_step": n, "nlay": NLAY5, "icld": 3,
                       "idrv": 1},
            "cpu_baseline": {"value": v, "unit": "columns/s", "cores": cores, "kind": "port",
                             "sample": f"{n} columns per step, {cores} threads; McICA sub-columns made beforehand"},
            "e2e": {"value": v, "unit": "columns/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- GPU arm
def traffic_from_profiles(name):
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("dram_bytes_per_launch_full_workload:"):
            return float(line.split(":")[1])
    return None


def fused_bytes_per_column(nlay: int, learned: bool) -> int:
    """Algorithmic bytes of the fused-cloud column kernel: every layer input
    (12 gas/state + cldfrac, ciwp, clwp, 2 radii, 16 aerosol, 16 tauc = 49 per
    layer), plev/tlev, tsfc, 16 emis, the 140 McICA draws and every output once;
    with the learned gas optics also the network's 280 binary16 outputs and flag
    per layer."""
    b = 8 * (49 * nlay + 2 * (nlay + 1) + 17) + 8 * GB_NGPT + 8 * (6 * (nlay + 1) + 2 * nlay)
    if learned:
        b += nlay * (280 * 2 + 1)
    return b


GB_NGPT = 140


class Workload:
    """Device arrays of the headline workload: a base grid shared by the
    members (pressure, gases, clouds, emissivity, aerosol, tauc) and per-member
    T/H2O and outputs, Fortran layout with leading dimension nbase."""

    SHARED = ("play", "plev", "tlev", "tsfc", "o3vmr", "co2vmr", "ch4vmr", "n2ovmr", "o2vmr", "cfc11vmr",
              "cfc12vmr", "cfc22vmr", "ccl4vmr", "emis", "tauaer", "cldfrac", "ciwp", "clwp", "rei", "rel", "tauc")

    def __init__(self, dev, nbase, nlay, nmem, seed, tile=TILE):
        import torch
        from brams_gb300.profiles import ProfileSpec, make_state
        from brams_gb300.tables_io import read_tables

        self.nbase, self.nlay, self.nmem, self.seed = nbase, nlay, nmem, seed
        tile = min(tile, nbase)
        st = make_state(ProfileSpec(ncol=tile, nlay=nlay, seed=seed, ptop=PTOP5, t_noise=4.0, h2o_sigma=0.5))
        tabs = read_tables(os.path.join(ROOT, "brams_gb300", "data", "lw_ref_tables.gblw"))
        st["tauc"] = cldprop_numpy(st, tabs)
        self.tile = st
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        rep = (nbase + tile - 1) // tile

        def up(a):  # Fortran (tile, ...) -> device tensor with memory order = Fortran (nbase, ...)
            t = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)).to(dev)
            return torch.cat([t] * rep, dim=-1)[..., :nbase].contiguous()

        d = {k: up(st[k]) for k in self.SHARED if k != "tauc"}
        tc = torch.from_numpy(np.ascontiguousarray(np.asarray(st["tauc"]).T)).to(dev)  # (nlay, tile, 16)
        d["tauc"] = torch.cat([tc] * rep, dim=1)[:, :nbase, :].contiguous()
        tl, hv = up(st["tlay"]), up(st["h2ovmr"])
        # one perturbation per replica of the tile ...
        tl += torch.randn(tl.shape, generator=g, device=dev, dtype=torch.float64)
        hv *= torch.exp(0.2 * torch.randn(hv.shape, generator=g, device=dev, dtype=torch.float64))
        self.d = d
        self.mem = []
        for m in range(nmem):  # ... and one per member
            t = tl + torch.randn(tl.shape, generator=g, device=dev, dtype=torch.float64)
            h = (hv * torch.exp(0.2 * torch.randn(hv.shape, generator=g, device=dev, dtype=torch.float64))).clamp_(3.0e-6, 0.05)
            o = {k: torch.zeros((nlay + 1, nbase), dtype=torch.float64, device=dev)
                 for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt")}
            o["hr"] = torch.zeros((nlay, nbase), dtype=torch.float64, device=dev)
            o["hrc"] = torch.zeros((nlay, nbase), dtype=torch.float64, device=dev)
            self.mem.append({"tlay": t, "h2ovmr": h, **o})
        del tl, hv

    def seed0(self, m):
        return self.seed * 1000003 + m * self.nbase

    def desc(self, m, c0=0, n=None, **extra):
        """Grid descriptor of member m, columns c0 .. c0+n-1 (pointer offsets, leading dimension nbase)."""
        from brams_gb300 import rrtmg_lw as R

        n = self.nbase - c0 if n is None else n
        arrays = {}
        for k, t in list(self.d.items()) + list(self.mem[m].items()):
            arrays[k] = t.data_ptr() + 8 * c0 * (16 if k == "tauc" else 1)
        arrays["reicmcl"], arrays["relqmcl"] = arrays["rei"], arrays["rel"]
        arrays.update(extra)
        return R.grid_desc(n, self.nlay, arrays, icld=3, cloud_mode=R.CLOUD_FUSED, seed0=self.seed0(m) + c0,
                           ld_in=self.nbase, ld_out=self.nbase)

    def host_columns(self, m, c0, n):
        """Inputs of member m, columns c0 .. c0+n-1, as Fortran numpy arrays (for the oracle)."""
        out = {}
        for k, t in list(self.d.items()) + [(k, self.mem[m][k]) for k in ("tlay", "h2ovmr")]:
            if k == "tauc":
                out[k] = np.asfortranarray(t[:, c0:c0 + n, :].cpu().numpy().T)
            else:
                out[k] = np.asfortranarray(t[..., c0:c0 + n].cpu().numpy().T)
        return out

    def outputs(self, m, c0, n):
        return {k: np.asfortranarray(self.mem[m][k][:, c0:c0 + n].cpu().numpy().T) for k in
                ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt", "hr", "hrc")}


def surrogate_step(ctx, mlp, wl, bufs, stream, ev=None):
    """One step of the learned path: per chunk, inference for the members then one batched column launch."""
    tau, frac, flag = bufs
    nch = 0
    for c0 in range(0, wl.nbase, CHUNK):
        n = min(CHUNK, wl.nbase - c0)
        grids = []
        for m in range(wl.nmem):
            r0 = m * CHUNK * wl.nlay
            sur = dict(sur_tau=tau[r0:].data_ptr(), sur_frac=frac[r0:].data_ptr(), sur_flag=flag[r0:].data_ptr())
            g = wl.desc(m, c0, n)
            mlp.infer(g, sur["sur_tau"], sur["sur_frac"], sur["sur_flag"], stream=stream)
            grids.append(wl.desc(m, c0, n, **sur))
        if ev is not None:
            ev[nch][0].record()
        ctx.rrtmg_lw_batch_device(grids, stream=stream)
        if ev is not None:
            ev[nch][1].record()
        nch += 1
    return nch


def log(msg):
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def gpu_arm(args, rank, world):
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from brams_gb300.build import build
    from brams_gb300 import rrtmg_lw as R
    from brams_gb300 import surrogate as S

    if rank == 0 or world == 1:
        build()
    if world > 1:
        torch.distributed.barrier()
        build()
    ctx = R.Context(device=local)
    stream = torch.cuda.current_stream(dev).cuda_stream
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    hbm = float(peaks.get("hbm_gbs", 6800.0))

    # ---------------- the learned gas optics
    wpath = S.DEFAULT_WEIGHTS
    if os.path.exists(wpath):
        mlp = R.Mlp(ctx, path=wpath)
        trained = "loaded " + os.path.relpath(wpath, ROOT)
    else:
        mlp, info = S.train(ctx, log=lambda *a: None)
        trained = f"trained in this run ({info['train_s']:.1f} s on {info['rows']} layers)"

    # ---------------- headline workload
    log("network ready; building the workload")
    nbase = args.nbase
    # the job is world x NMEM members; the library's shard plan (balanced by
    # layers, contiguous) gives this rank its members
    from brams_gb300.shard import shard_plan

    plan = shard_plan([(nbase, NLAY5)] * (NMEM * world), world, rank)
    mine = [i for i, (a, b) in enumerate(plan) if b > a]
    if len(mine) != NMEM or any(plan[i] != (0, nbase) for i in mine):
        raise RuntimeError(f"shard plan does not give rank {rank} whole members: {plan}")
    seed = BASE_SEED + 7919 * (mine[0] // NMEM)
    wl = Workload(dev, nbase, NLAY5, NMEM, seed)
    ncol = nbase * NMEM
    rows = CHUNK * NLAY5 * NMEM
    bufs = (torch.empty((rows, GB_NGPT), dtype=torch.float16, device=dev),
            torch.empty((rows, GB_NGPT), dtype=torch.float16, device=dev),
            torch.empty(rows, dtype=torch.uint8, device=dev))
    plain = lambda: ctx.rrtmg_lw_batch_device([wl.desc(m) for m in range(NMEM)], stream=stream)
    sur = lambda ev=None: surrogate_step(ctx, mlp, wl, bufs, stream, ev)
    torch.cuda.synchronize()
    log(f"workload on the device ({torch.cuda.memory_allocated(dev) / 1e9:.1f} GB); tuning")
    # launch shapes from the autotuner, for both kinds of batch, on a sample of the workload
    if args.no_tune:
        tuned = {"plain": ctx.tuning(NLAY5, R.KIND_FUSED), "learned": ctx.tuning(NLAY5, R.KIND_FUSED | R.KIND_LEARNED)}
    else:
        tuned = {"plain": ctx.autotune([wl.desc(m) for m in range(NMEM)], sample_cols=4 * CHUNK, reps=2, stream=stream)}
        report = {"plain": ctx.autotune_report()}
        n0 = min(CHUNK, nbase)
        g0 = []
        for m in range(NMEM):
            r0 = m * CHUNK * NLAY5
            ex = dict(sur_tau=bufs[0][r0:].data_ptr(), sur_frac=bufs[1][r0:].data_ptr(), sur_flag=bufs[2][r0:].data_ptr())
            mlp.infer(wl.desc(m, 0, n0), ex["sur_tau"], ex["sur_frac"], ex["sur_flag"], stream=stream)
            g0.append(wl.desc(m, 0, n0, **ex))
        tuned["learned"] = ctx.autotune(g0, sample_cols=0, reps=2, stream=stream)  # a whole chunk
        report["learned"] = ctx.autotune_report()
        log("autotuner candidates (variant, blocks/SM, ms): " + json.dumps(
            {k: [(c["variant"], c["blocks_per_sm"], round(c["ms"], 2)) for c in v] for k, v in report.items()}))

    def timed(fn, steps, evs=False):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        return e0.elapsed_time(e1) / 1e3 / steps

    log(f"tuned: {tuned}; timing the plain path")
    for _ in range(args.warmup):
        plain()
    t_plain = timed(plain, args.steps)
    log("timing the learned path")
    plain_out = wl.outputs(0, nbase // 2, SAMPLE)
    for _ in range(args.warmup):
        sur()
    if ctx.sync_status(stream) != 0:
        raise RuntimeError("column status nonzero on the benchmark inputs")
    nch = (nbase + CHUNK - 1) // CHUNK
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nch * args.steps)]
    with ClockSampler(local) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        e0.record()
        for k in range(args.steps):
            sur(ev[k * nch:(k + 1) * nch])
        e1.record()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
    t_sur = e0.elapsed_time(e1) / 1e3 / args.steps
    t_kernel = sum(a.elapsed_time(b) for a, b in ev) / 1e3 / len(ev)  # one column-kernel launch (with its draws)
    status = ctx.sync_status(stream)
    sur_out = wl.outputs(0, nbase // 2, SAMPLE)
    launches_per_step = nch * (2 * NMEM + 2)  # per chunk: inference and McICA draws per member, learned-only + hand-over kernels

    # ---------------- accuracy against the FP64 oracle
    log("accuracy against the oracle")
    acc = {}
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle

        pyoracle.build(tuned=True)
        c0 = nbase // 2
        st = wl.host_columns(0, c0, SAMPLE)
        mc = pyoracle.mcica_per_column(st, st["tauc"], icld=3, base_seed=wl.seed0(0) + c0)
        ref = pyoracle.rrtmg_lw(st, mc, nthreads=os.cpu_count() or 1, tuned=True)
        for name, o in (("surrogate", sur_out), ("plain", plain_out)):
            acc[name] = {"hr_rmse_k_per_day": float(np.sqrt(np.mean((o["hr"] - ref["hr"]) ** 2))),
                         "hr_max_k_per_day": float(np.abs(o["hr"] - ref["hr"]).max()),
                         "flux_rmse_w_m2": float(np.sqrt(np.mean(np.concatenate(
                             [(o[k] - ref[k]).ravel() ** 2 for k in ("uflx", "dflx")])))),
                         "flux_max_w_m2": float(max(np.abs(o[k] - ref[k]).max() for k in ("uflx", "dflx")))}
        acc["sample"] = f"{SAMPLE} contiguous columns of member 0 from column {c0}; FP64 oracle with the same seeds"

    # ---------------- e2e: every step's inputs from page-locked host memory, outputs back
    log("e2e")
    e2e = e2e_headline(ctx, mlp, wl, dev, stream, min(args.steps, 2), world, bufs)

    # operations per column the oracle counts, on a few columns of member 0
    c0 = nbase // 2
    st_f = wl.host_columns(0, c0, 16)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    flops_sample = counted_flops(st_f, pyoracle.mcica_per_column(st_f, st_f["tauc"], icld=3, base_seed=wl.seed0(0) + c0))

    # ---------------- batched nested grids (CUDA graph) and the network at 512x512x45
    log("batched grids")
    batched = None if args.no_batched else batched_block(ctx, dev, stream, args, hbm)
    log("network evaluation at 512x512x45")
    ev = None if args.no_batched else eval_block(ctx, mlp, dev, stream, args)
    log("non-McICA driver at 360x300x45")
    nomc = None if args.no_batched else nomcica_block(ctx, dev, stream, args)
    log("shortwave at 360x300x45")
    sw = None if args.no_sw else sw_block(ctx, dev, stream, args)

    # ---------------- drop-in block (ABI mode, 360x300x45)
    log("drop-in block")
    abi = None if args.no_abi else abi_block(ctx, dev, stream, args, rank, world, hbm)

    times = torch.tensor([t_sur, t_plain, t_kernel, e2e["t"]], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(times, op=torch.distributed.ReduceOp.MAX)
    t_sur, t_plain, t_kernel, t_e2e = (float(x) for x in times)
    if rank != 0:
        return
    alg = fused_bytes_per_column(NLAY5, True) * NMEM * min(CHUNK, nbase)
    achieved = alg / t_kernel / 1e9
    traffic = traffic_from_profiles("lw_rt_kernel_learned_traffic.txt")
    line = {
        "metric": METRIC, "value": world * ncol / t_sur, "unit": "columns/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_sur * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64acc (network bf16/fp32acc)", "data": "synthetic",
        "config": {"workload": f"surrogate + batched at scale: {NX}x{NY} columns x {NLAY5} layers (1000 -> 5 hPa) "
                               f"x {NMEM} ensemble members" if nbase == NX * NY else
                               f"reduced: {nbase} columns x {NLAY5} layers x {NMEM} members",
                   "columns_per_gpu": ncol, "nlay": NLAY5, "members": NMEM, "icld": 3, "idrv": 1,
                   "parallelism": f"{world} GPU(s), members of the {world * NMEM}-member job split by "
                                  "gb_rrtmg_lw_shard_plan (no collective on the data path)",
                   "clouds": "McICA generated in the kernel, MT19937 seed = base + column",
                   "gas_optics": "learned (MLP, " + trained + "), taumol for layers outside the training range",
                   "chunk_columns_per_member": CHUNK,
                   "launch_shapes": {k: {f: v[f] for f in ("threads", "min_blocks", "blocks_per_sm")}
                                     for k, v in tuned.items()},
                   "inference": "tcgen05 (tensor memory accumulators)",
                   "l2": "inputs (~90 GB per step) larger than L2; no flush",
                   "precision": "fp32 transfer, fp64 flux sums and heating rates; network bf16 with fp32 accumulation"},
        "plain_gpu": {"value": world * ncol / t_plain, "unit": "columns/s", "ms_per_step": t_plain * 1e3,
                      "speedup_of_surrogate": t_plain / t_sur},
        "accuracy": acc,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic,
                     # what DRAM actually moved (ncu bytes per launch over this run's launch time)
                     "dram_gbs": traffic / t_kernel / 1e9 if traffic else None,
                     "dram_frac": traffic / t_kernel / 1e9 / hbm if traffic else None,
                     "kernel": "lw_rt_kernel (transfer on the network's gas optics, fused clouds), one launch = 4 "
                               f"members x {min(CHUNK, nbase)} columns; alg bytes/column {fused_bytes_per_column(NLAY5, True)}",
                     "alg_bytes_per_launch": alg, "launch_ms": t_kernel * 1e3,
                     "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                     "fp32": fp32_roofline(flops_sample, ("inatm", "cldprmc", "rtrnmc"),
                                           NMEM * min(CHUNK, nbase), t_kernel)},
        "e2e": {"value": world * ncol / t_e2e, "unit": "columns/s", "h2d_bytes_per_step": e2e["h2d"],
                "d2h_bytes_per_step": e2e["d2h"], "host_data": e2e["note"],
                "host_path_matches_device_path": e2e["matches"]},
        "gpu_launches": launches_per_step * args.steps, "clocks": clk.summary(), "column_status": status,
    }
    if abi is not None:
        line["plain_abi"] = abi
    if batched is not None:
        line["batched"] = batched
    if ev is not None:
        line["eval"] = ev
    if nomc is not None:
        line["nomcica"] = nomc
    if sw is not None:
        line["shortwave"] = sw
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_headline(wl)
        line["cpu_configs"] = cpu_configs()
    print(json.dumps(line), flush=True)


def e2e_headline(ctx, mlp, wl, dev, stream, steps, world, bufs):
    """Surrogate path with host-resident inputs: per chunk, every input array of
    the four members is copied from page-locked host memory (the generator
    tile's columns, stored chunk by chunk so that every copy is one contiguous
    DMA), solved, and every output is copied back to page-locked memory.  The
    band cloud optical depths are not copied: cldprop runs on the device from
    the layer cloud state, as BRAMS would call it before McICA.  Chunks are
    pipelined over three staging buffers and three streams: the host-to-device
    copies of chunk i+1 and the device-to-host copies of chunk i-1 run while
    chunk i is solved (events order every reuse of a buffer).  Three staging
    buffers rather than two let a late copy of one chunk overlap two solves."""
    import torch
    from brams_gb300 import rrtmg_lw as R

    nlay, C = wl.nlay, min(CHUNK, wl.nbase)
    tile = wl.tile
    T = tile["play"].shape[0]
    nt = max(1, T // C)
    names = [k for k in wl.SHARED if k != "tauc"] + ["tlay", "h2ovmr"]
    host = {}
    for k in names:
        a = np.ascontiguousarray(np.asarray(tile[k], dtype=np.float64).T)  # (..., T)
        host[k] = [torch.from_numpy(np.ascontiguousarray(a[..., j * C:(j + 1) * C])).pin_memory() for j in range(nt)]
    outs = ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt", "hr", "hrc")
    NBUF = 3
    stage = []
    for _ in range(NBUF):
        members = []
        for m in range(wl.nmem):
            d = {k: torch.empty(host[k][0].shape, dtype=torch.float64, device=dev) for k in host}
            d["tauc"] = torch.empty((nlay, C, 16), dtype=torch.float64, device=dev)  # (16, C, nlay) Fortran
            for k in outs:
                d[k] = torch.empty((nlay + (0 if k in ("hr", "hrc") else 1), C), dtype=torch.float64, device=dev)
            members.append(d)
        stage.append(members)
    hout = [{k: torch.empty((wl.nmem,) + tuple(stage[0][0][k].shape), dtype=torch.float64).pin_memory() for k in outs}
            for _ in range(NBUF)]
    tau, frac, flag = bufs
    counts = {"h2d": 0, "d2h": 0}
    solve = torch.cuda.current_stream(dev)  # the stream the library calls run on
    assert solve.cuda_stream == stream
    s_in, s_cp, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    ev_in = [torch.cuda.Event() for _ in range(NBUF)]
    ev_cp = [torch.cuda.Event() for _ in range(NBUF)]
    ev_solved = [torch.cuda.Event() for _ in range(NBUF)]
    ev_out = [torch.cuda.Event() for _ in range(NBUF)]

    def step():
        h2d = d2h = 0
        for i, c0 in enumerate(range(0, wl.nbase, C)):
            j, b = i % nt, i % NBUF
            with torch.cuda.stream(s_in):
                if i >= NBUF:
                    s_in.wait_event(ev_solved[b])  # chunk i-2 has consumed these inputs
                for m in range(wl.nmem):
                    for k in host:
                        stage[b][m][k].copy_(host[k][j], non_blocking=True)
                        h2d += host[k][j].numel() * 8
                ev_in[b].record(s_in)
            # band cloud optical depths of the chunk on a stream of their own, so
            # that they overlap the solve of the chunk before without holding up
            # the copies of the next
            with torch.cuda.stream(s_cp):
                s_cp.wait_event(ev_in[b])
                for m in range(wl.nmem):
                    d = stage[b][m]
                    ctx.cldprop_lw_device(C, nlay, {"cldfrac": d["cldfrac"], "ciwp": d["ciwp"], "clwp": d["clwp"],
                                                    "rei": d["rei"], "rel": d["rel"], "taucloud": d["tauc"]},
                                          inflag=2, iceflag=3, liqflag=1, ld=C, stream=s_cp.cuda_stream)
                ev_cp[b].record(s_cp)
            solve.wait_event(ev_cp[b])
            if i >= NBUF:
                solve.wait_event(ev_out[b])  # chunk i-2's outputs have been read back
            grids = []
            for m in range(wl.nmem):
                d = stage[b][m]
                arrays = dict(d)
                arrays["reicmcl"], arrays["relqmcl"] = d["rei"], d["rel"]
                r0 = m * C * nlay
                g = R.grid_desc(C, nlay, arrays, icld=3, cloud_mode=R.CLOUD_FUSED, seed0=wl.seed0(m) + c0)
                mlp.infer(g, tau[r0:].data_ptr(), frac[r0:].data_ptr(), flag[r0:].data_ptr(), stream=stream)
                arrays.update(sur_tau=tau[r0:].data_ptr(), sur_frac=frac[r0:].data_ptr(), sur_flag=flag[r0:].data_ptr())
                grids.append(R.grid_desc(C, nlay, arrays, icld=3, cloud_mode=R.CLOUD_FUSED, seed0=wl.seed0(m) + c0))
            ctx.rrtmg_lw_batch_device(grids, stream=stream)
            ev_solved[b].record(solve)
            with torch.cuda.stream(s_out):
                s_out.wait_event(ev_solved[b])
                for m in range(wl.nmem):
                    for k in outs:
                        hout[b][k][m].copy_(stage[b][m][k], non_blocking=True)
                        d2h += stage[b][m][k].numel() * 8
                ev_out[b].record(s_out)
        torch.cuda.synchronize(dev)
        counts["h2d"], counts["d2h"] = h2d, d2h

    step()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    t = (time.perf_counter() - t0) / steps
    # the pipelined leg's last chunk, member 0, read back from host memory,
    # against the same inputs solved again without the pipeline
    nchunk = (wl.nbase + C - 1) // C
    il = nchunk - 1
    jl, bl, c0l = il % nt, il % NBUF, il * C
    d = {k: host[k][jl].to(dev) for k in host}
    d["tauc"] = torch.empty((nlay, C, 16), dtype=torch.float64, device=dev)
    for k in outs:
        d[k] = torch.empty((nlay + (0 if k in ("hr", "hrc") else 1), C), dtype=torch.float64, device=dev)
    ctx.cldprop_lw_device(C, nlay, {"cldfrac": d["cldfrac"], "ciwp": d["ciwp"], "clwp": d["clwp"], "rei": d["rei"],
                                    "rel": d["rel"], "taucloud": d["tauc"]}, inflag=2, iceflag=3, liqflag=1, ld=C,
                          stream=stream)
    arrays = dict(d)
    arrays["reicmcl"], arrays["relqmcl"] = d["rei"], d["rel"]
    g = R.grid_desc(C, nlay, arrays, icld=3, cloud_mode=R.CLOUD_FUSED, seed0=wl.seed0(0) + c0l)
    mlp.infer(g, tau.data_ptr(), frac.data_ptr(), flag.data_ptr(), stream=stream)
    arrays.update(sur_tau=tau.data_ptr(), sur_frac=frac.data_ptr(), sur_flag=flag.data_ptr())
    ctx.rrtmg_lw_batch_device([R.grid_desc(C, nlay, arrays, icld=3, cloud_mode=R.CLOUD_FUSED,
                                           seed0=wl.seed0(0) + c0l)], stream=stream)
    torch.cuda.synchronize(dev)
    matches = all(torch.equal(d[k].cpu(), hout[bl][k][0]) for k in outs)
    return {"t": t, "h2d": counts["h2d"], "d2h": counts["d2h"], "matches": matches,
            "note": f"every chunk copies all inputs of {wl.nmem} members x {C} columns from page-locked host memory "
                    f"(the generator tile's columns; the band cloud optical depths made on the device by cldprop on the copy stream) and "
                    f"reads all outputs back, pipelined over three staging buffers (copies of neighbouring chunks "
                    f"overlap the solve); {steps} timed steps"}


def cpu_baseline_headline(wl, seconds: float = 12.0, max_cols: int = 16384):
    """The FP64 oracle on all host cores over a bounded sample of member 0's
    columns (at most max_cols, whose McICA sub-columns take 268 KB each),
    repeated until about `seconds` of work."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build(tuned=True)
    cores = os.cpu_count() or 1
    n = min(wl.nbase, max_cols)
    st = wl.host_columns(0, 0, n)
    mc = pyoracle.mcica_per_column(st, st["tauc"], icld=3, base_seed=wl.seed0(0))
    done, t0 = 0, time.perf_counter()
    while True:
        pyoracle.rrtmg_lw(st, mc, nthreads=cores, tuned=True)
        done += n
        dt = time.perf_counter() - t0
        if dt >= seconds:
            break
    return {"value": done / dt, "unit": "columns/s", "cores": cores, "kind": "port",
            "sample": f"the first {n} columns of member 0 of the {NX}x{NY}x{NLAY5} workload, {done // n} passes "
                      f"({dt:.1f} s), {cores} threads, FP64 C++ restatement (-O3, Neoverse V2 tuning on aarch64); McICA sub-columns made "
                      "beforehand, not timed"}


def fp32_roofline(flops: dict, phases, columns: int, seconds: float) -> dict:
    """Counted operations of `phases` per column times the columns of one
    launch, over the launch time, against the nominal FP32 peak."""
    per_col = sum(flops[p] for p in phases)
    tf = per_col * columns / seconds / 1e12
    return {"bound": "fp32", "achieved": tf, "peak": FP32_PEAK_TFLOPS, "unit": "TFLOP/s", "frac": tf / FP32_PEAK_TFLOPS,
            "flops_per_column": per_col, "phases": list(phases),
            "peak_source": "nominal: 152 SMs x 128 lanes x 2 (FMA) x 2.07 GHz",
            "counted_by": "oracle/flop_count.h (additions, subtractions, multiplications, divisions of the FP64 restatement)"}


def _perturbed_members(base, members, gen, dev):
    """Ensemble members of a device grid: T + N(0, 1 K) and H2O x lognormal(0, 0.2) per (column, layer)."""
    import torch

    from brams_gb300 import surrogate as S

    out = []
    for _ in range(members):
        m = S.DeviceGrid.__new__(S.DeviceGrid)
        m.ncol, m.nlay = base.ncol, base.nlay
        m.d = {k: v.clone() for k, v in base.d.items()}
        m.d["tlay"] += torch.randn(m.d["tlay"].shape, generator=gen, device=dev, dtype=torch.float64)
        m.d["h2ovmr"] = (m.d["h2ovmr"] * torch.exp(0.2 * torch.randn(m.d["h2ovmr"].shape, generator=gen, device=dev,
                                                                     dtype=torch.float64))).clamp_(3.0e-6, 0.05)
        out.append(m)
    return out


def _host_of(m, n):
    """The first n columns of a device grid's inputs as Fortran numpy arrays (for the oracle)."""
    st = {}
    for k, t in m.d.items():
        if k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt", "hr", "hrc"):
            continue
        a = t.cpu().numpy()
        st[k] = np.asfortranarray(a[:, :n, :].T if k == "tauc" else a[..., :n].T)
    return st


def _errors(got, ref, n):
    return {"hr_rmse_k_per_day": float(np.sqrt(np.mean((got["hr"][:n] - ref["hr"]) ** 2))),
            "hr_max_k_per_day": float(np.abs(got["hr"][:n] - ref["hr"]).max()),
            "flux_max_w_m2": float(max(np.abs(got[k][:n] - ref[k]).max() for k in ("uflx", "dflx")))}


def batched_block(ctx, dev, stream, args, hbm):
    """Three nested grids x 8 members in one persistent launch captured in a CUDA graph."""
    import torch

    from brams_gb300 import surrogate as S
    from brams_gb300.profiles import ProfileSpec, make_state
    from brams_gb300.tables_io import read_tables

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    tabs = read_tables(os.path.join(ROOT, "brams_gb300", "data", "lw_ref_tables.gblw"))
    shapes = [(200, 180, 45), (150, 150, 45), (97, 97, 38)]
    members = 8
    gen = torch.Generator(device=dev)
    gen.manual_seed(BASE_SEED + 17)
    grids, seeds = [], []
    for gi, (nx, ny, nlay) in enumerate(shapes):
        st = make_state(ProfileSpec(ncol=nx * ny, nlay=nlay, seed=BASE_SEED + 31 * gi, ptop=PTOP, t_noise=4.0,
                                    h2o_sigma=0.5))
        base = S.DeviceGrid(st, cldprop_numpy(st, tabs))
        for m, mg in enumerate(_perturbed_members(base, members, gen, dev)):
            grids.append(mg)
            seeds.append((gi * members + m) * 100003 + BASE_SEED)
        del base
    descs = [g.desc(seed0=s) for g, s in zip(grids, seeds)]
    ncols = sum(g.ncol for g in grids)
    # tuned on the whole batch: a 65,536-column sample picked shapes up to 20% slower on the 543,272 columns
    best = ctx.autotune(descs, sample_cols=0, reps=2, stream=stream)
    graph = ctx.batch_graph(descs)
    try:
        for _ in range(args.warmup):
            graph.launch(stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            graph.launch(stream)
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / args.steps
    finally:
        graph.close()
    status = ctx.sync_status(stream)
    # oracle check: 512 columns of member 0 of the 45- and the 38-layer grid
    acc = {}
    for gi in (0, 2):
        m = grids[gi * members]
        st = _host_of(m, 512)
        mc = pyoracle.mcica_per_column(st, st["tauc"], icld=3, base_seed=seeds[gi * members])
        ref = pyoracle.rrtmg_lw(st, mc, nthreads=os.cpu_count() or 1, tuned=True)
        acc[f"grid{gi}_member0"] = _errors(m.outputs(), ref, 512)
    alg = sum(fused_bytes_per_column(g.nlay, False) * g.ncol for g in grids)
    st45 = _host_of(grids[0], 16)
    fl45 = counted_flops(st45, pyoracle.mcica_per_column(st45, st45["tauc"], icld=3, base_seed=seeds[0]))
    st38 = _host_of(grids[2 * members], 16)
    fl38 = counted_flops(st38, pyoracle.mcica_per_column(st38, st38["tauc"], icld=3, base_seed=seeds[2 * members]))
    flops = sum((fl38 if g.nlay == 38 else fl45)["total"] * g.ncol for g in grids)
    tf = flops / t / 1e12
    return {"workload": "batched uneven grids 200x180x45 + 150x150x45 + 97x97x38, x 8 members (T + N(0,1 K), "
                        "H2O x lognormal(0,0.2)), one persistent launch of taumol + transfer captured in a CUDA graph; "
                        "McICA clouds in the kernel; autotuned launch shape",
            "columns": ncols, "value": ncols / t, "unit": "columns/s", "ms_per_step": t * 1e3,
            "launch_shape": {k: best[k] for k in ("threads", "min_blocks", "blocks_per_sm")},
            "roofline": {"bound": "hbm", "achieved": alg / t / 1e9, "peak": hbm, "unit": "GB/s",
                         "frac": alg / t / 1e9 / hbm, "alg_bytes_per_step": alg},
            "fp32": {"bound": "fp32", "achieved": tf, "peak": FP32_PEAK_TFLOPS, "unit": "TFLOP/s",
                     "frac": tf / FP32_PEAK_TFLOPS, "flops_per_column_45": fl45["total"], "flops_per_column_38": fl38["total"],
                     "peak_source": "nominal", "counted_by": "oracle/flop_count.h"},
            "accuracy": acc, "column_status": status}


def eval_block(ctx, mlp, dev, stream, args):
    """The learned gas optics on 512x512 columns x 45 layers against the plain path and the FP64 oracle."""
    import torch

    from brams_gb300 import surrogate as S
    from brams_gb300.profiles import make_state, workload_spec
    from brams_gb300.tables_io import read_tables

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    tabs = read_tables(os.path.join(ROOT, "brams_gb300", "data", "lw_ref_tables.gblw"))
    st = make_state(workload_spec("eval_512x512x45"))
    tauc = cldprop_numpy(st, tabs)
    ncol, nlay = st["play"].shape
    gl, gp = S.DeviceGrid(st, tauc), S.DeviceGrid(st, tauc)
    rows = ncol * nlay
    tau = torch.empty((rows, GB_NGPT), dtype=torch.float16, device=dev)
    frac = torch.empty_like(tau)
    flag = torch.empty(rows, dtype=torch.uint8, device=dev)
    seed0 = 77

    def learned():
        mlp.infer(gl.desc(seed0=seed0), tau, frac, flag, stream=stream)
        ctx.rrtmg_lw_batch_device([gl.desc(seed0=seed0, sur_tau=tau.data_ptr(), sur_frac=frac.data_ptr(),
                                           sur_flag=flag.data_ptr())], stream=stream)

    def plain():
        ctx.rrtmg_lw_batch_device([gp.desc(seed0=seed0)], stream=stream)

    res = {}
    for name, fn in (("learned", learned), ("plain", plain)):
        for _ in range(args.warmup):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        res[name] = {"value": ncol / (e0.elapsed_time(e1) / 1e3 / args.steps), "unit": "columns/s"}
    n = 2048
    sub = {k: np.asfortranarray(v[:n]) for k, v in st.items()}
    mc = pyoracle.mcica_per_column(sub, np.asfortranarray(tauc[:, :n]), icld=3, base_seed=seed0)
    ref = pyoracle.rrtmg_lw(sub, mc, nthreads=os.cpu_count() or 1, tuned=True)
    res["learned"].update(_errors(gl.outputs(), ref, n))
    res["plain"].update(_errors(gp.outputs(), ref, n))
    res["layers_on_network"] = float(flag.float().mean().item())
    res["speedup_of_learned"] = res["learned"]["value"] / res["plain"]["value"]
    res["workload"] = ("512x512 columns x 45 layers (T noise N(0,4 K), H2O x lognormal(0,0.5)), McICA in the kernel; "
                       f"errors against the FP64 oracle on the first {n} columns")
    res["column_status"] = ctx.sync_status(stream)
    return res


def nomcica_block(ctx, dev, stream, args):
    """The non-McICA driver (gb_rrtmg_lw_nomcica_device: cldprop, taumol and
    the transfer with random or maximum/random overlap) on 360x300x45
    device arrays, and its error against the FP64 oracle on 512 columns."""
    import torch

    from brams_gb300 import rrtmg_lw as R
    from brams_gb300.profiles import make_state, workload_spec

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    st = make_state(workload_spec("drop_in_360x300x45"))
    ncol, nlay = st["play"].shape

    def dv(a):
        return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)).to(dev)

    d = {k: dv(st[k]) for k in R.STATE_ORDER + ["tauaer", "cldfrac", "ciwp", "clwp", "rei", "rel"]}
    d["tauc_band"] = torch.zeros((nlay, ncol, 16), dtype=torch.float64, device=dev)
    for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt"):
        d[k] = torch.zeros((nlay + 1, ncol), dtype=torch.float64, device=dev)
    d["hr"] = torch.zeros((nlay, ncol), dtype=torch.float64, device=dev)
    d["hrc"] = torch.zeros((nlay, ncol), dtype=torch.float64, device=dev)
    res = {"workload": "rrtmg_lw of the non-McICA driver, 360x300 columns x 45 layers on device arrays "
                       "(cldprop + taumol + transfer per call); errors against the FP64 oracle on 512 columns"}
    n = 512
    sub = {k: np.asfortranarray(v[:n]) for k, v in st.items()}
    for icld, name in ((1, "random_overlap"), (2, "max_random_overlap")):
        call = lambda: ctx.rrtmg_lw_nomcica_device(ncol, nlay, d, stream=stream, icld=icld)  # noqa: E731
        for _ in range(args.warmup):
            call()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            call()
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / args.steps
        got = {k: d[k].cpu().numpy().T for k in ("uflx", "dflx", "hr")}
        ref = pyoracle.rrtmg_lw_nomcica(sub, icld, tuned=True)
        res[name] = {"value": ncol / t, "unit": "columns/s", "ms_per_step": t * 1e3, **_errors(got, ref, n)}
    res["column_status"] = ctx.sync_status(stream)
    return res


def sw_block(ctx, dev, stream, args):
    """RRTMG_SW on 360x300 columns x 45 layers of device arrays: McICA
    sub-columns (gb_mcica_subcol_sw_device, per-column seeds) and the
    solver (gb_rrtmg_sw_device) timed per step, its error against the FP64
    oracle on 256 columns, and the oracle's throughput on the host cores."""
    import ctypes as C

    import torch

    from brams_gb300 import rrtmg_lw as R
    from brams_gb300.profiles import make_state, workload_spec

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    ctx.sw_ini(1004.0)
    st = make_state(workload_spec("drop_in_360x300x45", ncol=args.sw_ncol))
    ncol, nlay = st["play"].shape
    rng = np.random.default_rng(2024)
    for k in ("asdir", "asdif", "aldir", "aldif"):
        st[k] = rng.uniform(0.05, 0.4, ncol)
    st["coszen"] = rng.uniform(0.05, 1.0, ncol)
    st["tauaer_sw"] = np.asfortranarray(rng.uniform(0.0, 0.05, (ncol, nlay, 14)))
    st["ssaaer_sw"] = np.asfortranarray(rng.uniform(0.8, 0.99, (ncol, nlay, 14)))
    st["asmaer_sw"] = np.asfortranarray(rng.uniform(0.5, 0.8, (ncol, nlay, 14)))
    band = {k: np.asfortranarray(rng.uniform(lo, hi, (14, ncol, nlay)))
            for k, lo, hi in (("tauc", 0.5, 10.0), ("ssac", 0.9, 1.0), ("asmc", 0.7, 0.9), ("fsfc", 0.0, 0.5))}

    def dv(a):
        return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)).to(dev)

    d = {k: dv(st[k]) for k in R.SW_STATE + ["tauaer_sw", "ssaaer_sw", "asmaer_sw", "cldfrac", "ciwp", "clwp",
                                             "rei", "rel"]}
    b = {k: dv(v) for k, v in band.items()}
    m = {k: torch.zeros((nlay, ncol, 112), dtype=torch.float64, device=dev)
         for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl", "ssacmcl", "asmcmcl", "fsfcmcl")}
    m["reicmcl"] = torch.zeros((nlay, ncol), dtype=torch.float64, device=dev)
    m["relqmcl"] = torch.zeros((nlay, ncol), dtype=torch.float64, device=dev)
    o = {k: torch.zeros((nlay + 1, ncol), dtype=torch.float64, device=dev) for k in ("swuflx", "swdflx", "swuflxc", "swdflxc")}
    o["swhr"] = torch.zeros((nlay, ncol), dtype=torch.float64, device=dev)
    o["swhrc"] = torch.zeros((nlay, ncol), dtype=torch.float64, device=dev)
    L = ctx.L
    seed0 = 5

    def mcica():
        ir = C.c_int(1)
        rc = L.gb_mcica_subcol_sw_device(ctx.h, stream, ncol, nlay, 3, seed0, C.byref(ir),
                                         *[d[k].data_ptr() for k in ("play", "cldfrac", "ciwp", "clwp", "rei", "rel")],
                                         *[b[k].data_ptr() for k in ("tauc", "ssac", "asmc", "fsfc")], None,
                                         *[m[k].data_ptr() for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "reicmcl",
                                                                     "relqmcl", "taucmcl", "ssacmcl", "asmcmcl",
                                                                     "fsfcmcl")], ncol, 1)
        assert rc == 0

    def solve():
        ic, ia = C.c_int(3), C.c_int(10)
        rc = L.gb_rrtmg_sw_device(ctx.h, stream, ncol, nlay, C.byref(ic), C.byref(ia),
                                  *[d[k].data_ptr() for k in R.SW_STATE], 1.0, 0, 1368.22, -1, 2, 3, 1,
                                  *[m[k].data_ptr() for k in R.SW_CLOUD],
                                  *[d[k].data_ptr() for k in ("tauaer_sw", "ssaaer_sw", "asmaer_sw")], None,
                                  *[o[k].data_ptr() for k in R.SW_OUT], ncol, ncol, None)
        assert rc == 0

    res = {"workload": "rrtmg_sw (McICA, icld 3, iaer 10, iceflag 3, liqflag 1), "
                       + ("360x300 columns" if ncol == NCOL else f"{ncol} columns") + " x 45 layers of "
                       "device arrays; mcica_subcol_sw on the device with per-column seeds; the solver in both "
                       "precisions of its column kernel: rrtmg_sw = fp32 gas optics, cloud optics and two-stream "
                       "solution with fp64 flux sums and heating rates (the default), rrtmg_sw_fp64 = fp64 "
                       "throughout"}

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / args.steps
        return {"value": ncol / t, "unit": "columns/s", "ms_per_step": t * 1e3}

    res["mcica_subcol_sw"] = timed(mcica)
    if args.no_cpu:  # both precisions timed, no oracle
        for name, bits in (("rrtmg_sw", 32), ("rrtmg_sw_fp64", 64)):
            ctx.sw_set_precision(bits)
            res[name] = timed(solve)
            res[name]["column_status"] = ctx.sync_status(stream)
        ctx.sw_set_precision(32)
        return res
    n = 256
    sub = {k: np.asfortranarray(v[:n]) for k, v in st.items()}
    mc = {k: np.asfortranarray(v.cpu().numpy().T[:, :n] if v.dim() == 3 else v.cpu().numpy().T[:n])
          for k, v in m.items()}
    ref = pyoracle.rrtmg_sw(sub, mc, icld=3, iaer=10, tuned=True, nthreads=os.cpu_count() or 1)
    # operations per column counted on the oracle's code path (64 of the sampled columns)
    cs = {k: np.asfortranarray(v[:64]) for k, v in sub.items()}
    cm = {k: np.asfortranarray(v[:, :64] if v.ndim == 3 else v[:64]) for k, v in mc.items()}
    flops = pyoracle.sw_flops_per_column(cs, cm, icld=3, iaer=10)
    for name, bits in (("rrtmg_sw", 32), ("rrtmg_sw_fp64", 64)):
        ctx.sw_set_precision(bits)
        res[name] = timed(solve)
        peak = FP32_PEAK_TFLOPS if bits == 32 else FP64_PEAK_TFLOPS
        ach = flops * res[name]["value"] / 1e12
        res[name]["roofline"] = {"bound": f"fp{bits}", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                                 "frac": ach / peak, "flops_per_column": flops, "peak_source": "nominal",
                                 "counted_by": "oracle/flop_count.h on the shortwave restatement (a division "
                                               "or square root counts as one operation)"}
        res[name]["column_status"] = ctx.sync_status(stream)
        got = {k: v.cpu().numpy().T[:n] for k, v in o.items()}
        res[name]["accuracy"] = {
            "flux_max_w_m2": float(max(np.abs(got[k] - ref[k]).max() for k in ("swuflx", "swdflx", "swuflxc",
                                                                               "swdflxc"))),
            "hr_max_k_per_day": float(max(np.abs(got[k] - ref[k]).max() for k in ("swhr", "swhrc"))),
            "hr_rmse_k_per_day": float(np.sqrt(np.mean((got["swhr"] - ref["swhr"]) ** 2))), "columns": n}
    ctx.sw_set_precision(32)
    # the FP64 oracle on the host cores, 4,096 columns of the same inputs
    nc = 4096
    sub = {k: np.asfortranarray(v[:nc]) for k, v in st.items()}
    mcs = {k: np.asfortranarray(v.cpu().numpy().T[:, :nc] if v.dim() == 3 else v.cpu().numpy().T[:nc])
           for k, v in m.items()}
    cores = os.cpu_count() or 1
    pyoracle.rrtmg_sw(sub, mcs, icld=3, iaer=10, tuned=True, nthreads=cores)
    t0, reps = time.perf_counter(), 0
    while reps < 3 or time.perf_counter() - t0 < 5.0:
        pyoracle.rrtmg_sw(sub, mcs, icld=3, iaer=10, tuned=True, nthreads=cores)
        reps += 1
    dt = time.perf_counter() - t0
    res["cpu_oracle"] = {"value": nc * reps / dt, "unit": "columns/s", "cores": cores, "kind": "port",
                         "sample": f"{nc} columns x {nlay} layers, {reps} passes ({dt:.1f} s)"}
    return res


def cpu_configs(seconds: float = 5.0) -> dict:
    """The FP64 oracle on all host cores: the 64x64x38 configuration in full
    and a sample of the 360x300x45 one (McICA sub-columns made beforehand)."""
    from brams_gb300.profiles import make_state, workload_spec

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build(tuned=True)
    cores = os.cpu_count() or 1
    out = {}
    for name, ncol in (("oracle_64x64x38", None), ("drop_in_360x300x45", 8192)):
        st = make_state(workload_spec(name, ncol=ncol))
        mc = pyoracle.mcica_per_column(st, pyoracle.cldprop_columns(st), icld=3, base_seed=1)
        n = st["play"].shape[0]
        done, reps, t0 = 0, 0, time.perf_counter()
        while reps < 3 or time.perf_counter() - t0 < seconds:
            pyoracle.rrtmg_lw(st, mc, nthreads=cores, tuned=True)
            done += n
            reps += 1
        dt = time.perf_counter() - t0
        out[name] = {"value": done / dt, "unit": "columns/s", "cores": cores, "kind": "port",
                     "sample": f"{n} columns x {st['play'].shape[1]} layers, {reps} passes ({dt:.1f} s)"}
    return out


def abi_block(ctx, dev, stream, args, rank, world, hbm):
    """Drop-in path: gb_rrtmg_lw_device on the reference's McICA arrays (360x300x45) and gb_rrtmg_lw on host buffers."""
    import torch
    from brams_gb300.rrtmg_lw import OUT_ORDER, STATE_ORDER

    ncol, nlay = args.abi_ncol, NLAY
    seed = BASE_SEED + rank * 7919
    st, tauc = make_inputs(ncol, nlay, seed)

    def dev_f(a):
        return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).to(dev)

    d = {k: dev_f(st[k]) for k in STATE_ORDER}
    d["tauaer"] = dev_f(st["tauaer"])
    for k in ("cldfrac", "ciwp", "clwp", "rei", "rel"):
        d[k] = dev_f(st[k])
    d["tauc"] = dev_f(tauc)
    for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl"):
        d[k] = torch.empty((nlay, ncol, 140), dtype=torch.float64, device=dev)
    d["reicmcl"] = torch.empty((nlay, ncol), dtype=torch.float64, device=dev)
    d["relqmcl"] = torch.empty((nlay, ncol), dtype=torch.float64, device=dev)
    ctx.mcica_subcol_lw_device(ncol, nlay, d, icld=3, permuteseed=seed, irng=1, seed_per_column=True, stream=stream)
    for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt"):
        d[k] = torch.empty((nlay + 1, ncol), dtype=torch.float64, device=dev)
    d["hr"] = torch.empty((nlay, ncol), dtype=torch.float64, device=dev)
    d["hrc"] = torch.empty((nlay, ncol), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()

    def step():
        ctx.rrtmg_lw_device(ncol, nlay, d, stream=stream)

    # the autotuner picks the launch shape for this layer count and kind (caller sub-columns)
    shape = None
    if not args.no_tune:
        from brams_gb300 import rrtmg_lw as R
        shape = ctx.autotune([R.grid_desc(ncol, nlay, d, cloud_mode=R.CLOUD_SUBCOL)],
                             sample_cols=0, reps=2, stream=stream)  # the whole call: a sample tunes to its own size
    for _ in range(args.warmup):
        step()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    t_dev = e0.elapsed_time(e1) / 1e3 / args.steps
    status = ctx.sync_status(stream)
    host = {}
    ins = list(STATE_ORDER) + ["tauaer", "cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl", "reicmcl", "relqmcl"]
    for k in ins:
        h = torch.empty(d[k].shape, dtype=d[k].dtype, pin_memory=True)
        h.copy_(d[k])
        host[k] = h
    for k in OUT_ORDER:
        host[k] = torch.empty(d[k].shape, dtype=torch.float64, pin_memory=True)
    h2d = sum(host[k].numel() * 8 for k in ins)
    d2h = sum(host[k].numel() * 8 for k in OUT_ORDER)
    hp = {k: v.data_ptr() for k, v in host.items()}
    if ctx.rrtmg_lw_host_ptrs(ncol, nlay, hp) != 0:
        raise RuntimeError("gb_rrtmg_lw status nonzero")
    n = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(n):
        ctx.rrtmg_lw_host_ptrs(ncol, nlay, hp)
    t_e2e = (time.perf_counter() - t0) / n
    same = bool(torch.equal(host["hr"].to(dev), d["hr"]) and torch.equal(host["uflx"].to(dev), d["uflx"]))
    alg = abi_bytes_per_column(nlay) * ncol
    achieved = alg / t_dev / 1e9
    return {"workload": "rrtmg_lw drop-in (McICA arrays as the reference passes them), "
                        + ("360x300 columns x 45 layers" if ncol == NCOL else f"{ncol} columns x 45 layers"),
            "value": world * ncol / t_dev, "unit": "columns/s", "ms_per_step": t_dev * 1e3,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": traffic_from_profiles("lw_full_kernel_drop_in_traffic.txt"), "alg_bytes_per_launch": alg},
            "e2e": {"value": world * ncol / t_e2e, "unit": "columns/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "host_path_matches_device_path": same},
            "launch_shape": ({k: shape[k] for k in ("threads", "min_blocks", "blocks_per_sm")} if shape
                             else "default"),
            "column_status": status}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nbase", type=int, default=NX * NY, help="base-grid columns (each of the 4 members)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the oracle accuracy check and the CPU baseline")
    ap.add_argument("--no-abi", action="store_true", help="skip the 360x300x45 drop-in block")
    ap.add_argument("--no-tune", action="store_true", help="default launch shapes instead of the autotuner's")
    ap.add_argument("--abi-ncol", type=int, default=NCOL, help="columns of the drop-in block")
    ap.add_argument("--sw-ncol", type=int, default=NCOL, help="columns of the shortwave block")
    ap.add_argument("--no-sw", action="store_true", help="skip the shortwave block")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the nested-grid, 512x512x45 and non-McICA blocks")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "gloo" if args.impl == "reference" else "nccl"
        if backend == "nccl":
            import torch

            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend)
    try:
        if args.impl == "reference":
            reference_arm(args, rank, world)
        else:
            gpu_arm(args, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    main()
