"""Benchmark of the GB300 RRTMG_LW column solver.

One step = one pass of rrtmg_lw over the 360x300-column, 45-layer BRAMS-scale
workload (108,000 columns, McICA sub-columns with seed = base + column index,
FP32 gas optics and transfer with FP64 flux accumulation and heating rates).

  value  -- columns/s of the kernel on device-resident inputs
            (gb_rrtmg_lw_device, inputs already in HBM; 23 GB of inputs per
            step, far larger than the 129 MB L2, so no L2 flush is needed)
  e2e    -- columns/s through the reference-facing C ABI gb_rrtmg_lw with
            page-locked HOST buffers: host->device copies, kernel and
            device->host copies inside the timed region
  roofline -- the kernel's achieved algorithmic bandwidth against the
            measured HBM copy bandwidth; algorithmic bytes per column are
            8*(600*nlay + 25) (every rrtmg_lw input and output once)
  cpu_baseline -- the FP64 oracle (C++ restatement of the reference) on the
            host cores, on a bounded sample of the same columns

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
NCOL, NLAY, PTOP = 360 * 300, 45, 10.0
BASE_SEED = 1


def abi_bytes_per_column(nlay: int) -> int:
    return 8 * (600 * nlay + 25)


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
        pyoracle.build(native=True)
        native = True
    except Exception:
        native = False
    cores = os.cpu_count() or 1
    ncol = st["play"].shape[0]

    def sub(n):
        s = {k: np.asfortranarray(v[:n]) for k, v in st.items()}
        m = {k: np.asfortranarray(v[:, :n] if v.ndim == 3 else v[:n]) for k, v in mc.items()}
        return s, m

    probe = min(ncol, 64 * cores)
    s, m = sub(probe)
    t0 = time.perf_counter()
    pyoracle.rrtmg_lw(s, m, nthreads=cores, native=native)
    dt = time.perf_counter() - t0
    n = int(min(ncol, max(probe, probe * max_seconds / max(dt, 1e-6))))
    s, m = sub(n)
    t0 = time.perf_counter()
    pyoracle.rrtmg_lw(s, m, nthreads=cores, native=native)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "columns/s", "cores": cores, "kind": "port",
            "sample": f"first {n} of {ncol} columns of the 360x300x45 workload, one pass, "
                      f"{cores} threads, FP64 C++ restatement ({'-O3 native' if native else '-O2'})"}


def reference_arm(args, rank, world):
    """--impl reference: the CPU implementation alone, all host threads."""
    if rank != 0:
        return
    st, tauc = make_inputs(NCOL, NLAY, BASE_SEED)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build(native=True)
    cores = os.cpu_count() or 1
    n = min(NCOL, 2048 * cores // 4)
    s = {k: np.asfortranarray(v[:n]) for k, v in st.items()}
    mc = pyoracle.mcica_per_column(s, np.asfortranarray(tauc[:, :n]), icld=3, base_seed=BASE_SEED)
    for _ in range(args.warmup):
        pyoracle.rrtmg_lw(s, mc, nthreads=cores, native=True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pyoracle.rrtmg_lw(s, mc, nthreads=cores, native=True)
    dt = (time.perf_counter() - t0) / args.steps
    v = n / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "columns/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "rrtmg_lw 360x300 columns x 45 layers (sample per step)", "columns_per_step": n,
                       "nlay": NLAY, "icld": 3, "idrv": 1},
            "cpu_baseline": {"value": v, "unit": "columns/s", "cores": cores, "kind": "port",
                             "sample": f"{n} columns per step of the 360x300x45 workload"},
            "e2e": {"value": v, "unit": "columns/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- GPU arm
def traffic_from_profiles():
    path = os.path.join(ROOT, "profiles", "lw_column_kernel_c2_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("dram_bytes_per_launch_full_workload:"):
            return float(line.split(":")[1])
    return None


def gpu_arm(args, rank, world):
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from brams_gb300.build import build
    from brams_gb300.rrtmg_lw import Context, OUT_ORDER, STATE_ORDER

    if rank == 0 or world == 1:
        build()
    if world > 1:
        torch.distributed.barrier()
        build()
    ctx = Context(device=local)
    ncol, nlay = args.ncol, NLAY
    seed = BASE_SEED + rank * 7919
    st, tauc = make_inputs(ncol, nlay, seed)

    # device-resident inputs in the reference's Fortran layout
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
    stream = torch.cuda.current_stream(dev).cuda_stream
    ctx.mcica_subcol_lw_device(ncol, nlay, d, icld=3, permuteseed=seed, irng=1, seed_per_column=True, stream=stream)
    for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt"):
        d[k] = torch.empty((nlay + 1, ncol), dtype=torch.float64, device=dev)
    d["hr"] = torch.empty((nlay, ncol), dtype=torch.float64, device=dev)
    d["hrc"] = torch.empty((nlay, ncol), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()

    def step():
        ctx.rrtmg_lw_device(ncol, nlay, d, stream=stream)

    for _ in range(args.warmup):
        step()
    if ctx.sync_status(stream) != 0:
        raise RuntimeError("column status nonzero on the benchmark inputs")
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ev0.record()
        for _ in range(args.steps):
            step()
        ev1.record()
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t_dev = ev0.elapsed_time(ev1) / 1e3 / args.steps
    status = ctx.sync_status(stream)

    # e2e through the host-pointer C ABI with page-locked host buffers
    host = {}
    for k in list(STATE_ORDER) + ["tauaer", "cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl", "reicmcl", "relqmcl"]:
        t = d[k]
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t)
        host[k] = h
    for k in OUT_ORDER:
        host[k] = torch.empty(d[k].shape, dtype=torch.float64, pin_memory=True)
    h2d = sum(host[k].numel() * 8 for k in list(STATE_ORDER) + ["tauaer", "cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl", "reicmcl", "relqmcl"])
    d2h = sum(host[k].numel() * 8 for k in OUT_ORDER)
    hp = {k: v.data_ptr() for k, v in host.items()}
    rc = ctx.rrtmg_lw_host_ptrs(ncol, nlay, hp)
    if rc != 0:
        raise RuntimeError(f"gb_rrtmg_lw status {rc}")
    e2e_steps = max(1, min(args.steps, 5))
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        rc = ctx.rrtmg_lw_host_ptrs(ncol, nlay, hp)
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    # the host path must reproduce the device path bit for bit
    same = bool(torch.equal(host["hr"].to(dev), d["hr"]) and torch.equal(host["uflx"].to(dev), d["uflx"]))

    # cross-rank max of the per-step times
    times = torch.tensor([t_dev, t_e2e], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(times, op=torch.distributed.ReduceOp.MAX)
    t_dev, t_e2e = float(times[0]), float(times[1])
    if rank != 0:
        return
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    alg = abi_bytes_per_column(nlay) * ncol
    achieved = alg / t_dev / 1e9
    traffic = traffic_from_profiles()
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": world * ncol / t_dev, "unit": "columns/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_dev * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64acc", "data": "synthetic",
        "config": {"workload": "rrtmg_lw plain GPU path, 360x300 columns x 45 layers (BRAMS operational scale)",
                   "columns_per_gpu": ncol, "nlay": nlay, "icld": 3, "idrv": 1, "inflglw": 2, "iceflglw": 3,
                   "liqflglw": 1, "mcica": "140 sub-columns, MT19937 seed = base + column",
                   "l2": "inputs (23 GB per step) larger than L2; no flush", "precision":
                   "fp32 gas optics and transfer, fp64 flux accumulation and heating rates"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "alg_bytes_per_launch": alg,
                     "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"},
        "e2e": {"value": world * ncol / t_e2e, "unit": "columns/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "host_path_matches_device_path": same},
        "gpu_launches": args.steps, "clocks": clocks, "column_status": status,
    }
    if not args.no_cpu:
        mc_host = {k: host[k].numpy().T if host[k].dim() == 2 else np.transpose(host[k].numpy(), (2, 1, 0))
                   for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl", "reicmcl", "relqmcl")}
        mc_host = {k: np.asfortranarray(v) for k, v in mc_host.items()}
        line["cpu_baseline"] = cpu_baseline(st, mc_host)
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ncol", type=int, default=NCOL)
    ap.add_argument("--no-cpu", action="store_true")
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
