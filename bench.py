"""Throughput of the LBM solver step on GB300: MLUPs/s and its HBM-roofline fraction.

Workload (one GPU): D3Q19 TRT, FP32 arithmetic with FP16S DDF storage, 512x256x256 x-channel with
TYPE_E inlet/outlet planes at u=(0.075,0,0), rho=1, TYPE_S y/z walls and a TYPE_S|TYPE_X sphere of
radius 32 at (128,128,128); nu = 0.075*64/100 (Re=100 on the sphere diameter). Synthetic, seeded
geometry; the DDFs (1.27 GB) exceed L2 (129 MB), so no L2 flush is needed between steps.

A bench step is one LBM time step (one stream_collide launch over all 33.5M cells). ``value``
times K steps on the device with CUDA events on the solver's stream (inputs resident in HBM);
``e2e`` times the whole job through the public API from pinned host buffers: upload of
rho/u/flags, initialize, the same K steps, update_fields and download of rho/u.

``--impl reference`` times the reference's own kernel code on the host CPU (its OpenCL C text
compiled for the CPU where available, else the CPU restatement of the scheme) on the same
workload, over a bounded number of steps.

Under torchrun (N>1) every rank runs an independent replica of the workload on its own GPU
(the solver path is one domain per GPU; there is no data exchange to shard).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(name="sphere_channel_512x256x256_d3q19_trt_fp16s", Nx=512, Ny=256, Nz=256, q=19, collision="trt", storage="fp16s",
                extensions=("eq",), u_in=0.075, radius=32.0, center=(128.0, 128.0, 128.0), nu=0.075 * 64.0 / 100.0)
# the kernel the solver picks for this workload (fast arithmetic, FP16S storage, even Nx)
KERNEL = "k_stream_collide_pairs_pipe<19,FP16S,TRT,EQ> (two cells per thread, packed FP32x2, per-thread cp.async prefetch)"


def set_size(spec):
    """--size NXxNYxNZ: the same channel scaled (sphere radius and centre with Ny), for profiling captures."""
    Nx, Ny, Nz = (int(v) for v in spec.lower().split("x"))
    k = Ny / 256.0
    WORKLOAD.update(name=f"sphere_channel_{Nx}x{Ny}x{Nz}_d3q19_trt_fp16s", Nx=Nx, Ny=Ny, Nz=Nz, radius=32.0 * k,
                    center=(128.0 * k, 128.0 * k, 128.0 * k), nu=0.075 * 64.0 * k / 100.0)
METRIC = "MLUPs/s"
FALLBACK_HBM_GBS = 6800.0


def workload_fields():
    from fluidx3d_gb300 import setups as S
    w = WORKLOAD
    return S.sphere_channel(w["Nx"], w["Ny"], w["Nz"], u_in=w["u_in"], radius=w["radius"], center=w["center"])


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def traffic_per_launch():
    """DRAM bytes per stream_collide launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "stream_collide_traffic.json")
    if os.path.isfile(p):
        with open(p) as f:
            d = json.load(f)
        return d.get(WORKLOAD["name"])
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu_index, self.rows, self.proc = gpu_index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200",
                                          "-i", str(self.gpu_index)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for k, name in enumerate(names):
                if len(r) > 4 + k and r[4 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world <= 1:
        return None, 0, 1, 0
    import torch
    import torch.distributed as dist
    rank, local = int(os.environ["RANK"]), int(os.environ.get("LOCAL_RANK", "0"))
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return dist, rank, world, local


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline_run(K, time_budget_s=15.0, threads=None):
    """The reference's kernels (or the CPU restatement) on the host cores, same workload, bounded."""
    import oracle
    w = WORKLOAD
    threads = threads or os.cpu_count() or 1
    kind = "port"
    try:
        from oracle.ref_harness import build_ref
        built = build_ref.build_all([(w["q"], w["collision"], w["storage"], tuple(w["extensions"]))], jobs=1)
        if built:
            kind = "reference"
    except Exception:  # noqa: BLE001
        built = []
    cls = oracle.RefHarness if kind == "reference" else oracle.Oracle
    m = cls(w["Nx"], w["Ny"], w["Nz"], q=w["q"], collision=w["collision"], storage=w["storage"], extensions=w["extensions"], nu=w["nu"],
            threads=threads)
    f = workload_fields()
    m.rho[:], m.u[:], m.flags[:] = f["rho"], f["u"], f["flags"]
    m.initialize()
    m.run(1)  # warm-up step
    done, t0 = 0, time.perf_counter()
    while done < K:
        m.run(1)
        done += 1
        if time.perf_counter() - t0 > time_budget_s:
            break
    dt = time.perf_counter() - t0
    N = w["Nx"] * w["Ny"] * w["Nz"]
    return dict(value=N * done / dt / 1e6, unit=METRIC, cores=threads, kind=kind,
                sample=f"{done} full time steps of the {w['Nx']}x{w['Ny']}x{w['Nz']} workload ({'reference OpenCL C kernels compiled for the CPU' if kind == 'reference' else 'CPU restatement of the scheme'}), {threads} threads, {dt:.1f} s")


def run_reference_arm(args):
    dist, rank, world, _ = dist_setup(args.gpus)
    if rank != 0:
        return 0
    steps = args.steps
    r = cpu_baseline_run(steps, time_budget_s=max(10.0, min(120.0, 0.5 * steps)))
    w = WORKLOAD
    line = {"impl": "reference", "metric": METRIC, "value": r["value"], "unit": METRIC, "n_gpus": args.gpus, "steps": steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w["name"], "cells": w["Nx"] * w["Ny"] * w["Nz"], "velocity_set": "D3Q19", "collision": "TRT",
                       "ddf_storage": "FP16S", "device": "host CPU"},
            "cpu_baseline": {"value": r["value"], "unit": METRIC, "cores": r["cores"], "kind": r["kind"], "sample": r["sample"]},
            "e2e": {"value": r["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_gpu_arm(args):
    dist, rank, world, local = dist_setup(args.gpus)
    import torch
    from fluidx3d_gb300 import LBM, _capi as C
    w = WORKLOAD
    N = w["Nx"] * w["Ny"] * w["Nz"]
    f = workload_fields()
    lbm = LBM(w["Nx"], w["Ny"], w["Nz"], w["nu"], velocity_set=w["q"], collision=w["collision"], storage=w["storage"],
              extensions=w["extensions"], device=local)
    stream = torch.cuda.Stream(device=local)
    lbm._check(C.load().lbm_set_stream(lbm.handle, stream.cuda_stream))
    lbm.rho.data[:], lbm.u.data[:], lbm.flags.data[:] = f["rho"], f["u"], f["flags"]
    lbm.initialize()
    for _ in range(args.warmup):
        lbm.run(1)
    bpc = lbm.bandwidth_bytes_per_cell()
    K = args.steps
    # ---- device-resident throughput: K stream_collide launches bracketed by CUDA events on the solver's stream
    torch.cuda.synchronize(local)
    barrier(dist)
    torch.cuda.synchronize(local)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        start.record(stream)
        lbm.run(K)
        stop.record(stream)
        stop.synchronize()
    torch.cuda.synchronize(local)
    barrier(dist)
    ms = start.elapsed_time(stop)
    ms_max = max_over_ranks(dist, ms)
    value = world * N * K / (ms_max * 1e-3) / 1e6
    fluid = int(np.count_nonzero((f["flags"] & 3) != 1))  # cells the step updates (not TYPE_S)
    # ---- end-to-end job through the public API with pinned host buffers
    hb = {k: C.pinned_empty(f[k].shape, f[k].dtype) for k in ("rho", "u", "flags")}
    for k in hb:
        hb[k][:] = f[k]
    out_rho, out_u = C.pinned_empty((N,), np.float32), C.pinned_empty((3 * N,), np.float32)
    L = C.load()
    torch.cuda.synchronize(local)
    barrier(dist)
    t0 = time.perf_counter()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    lbm._check(L.lbm_write_field(lbm.handle, C.FIELD_RHO, hb["rho"].ctypes.data, hb["rho"].nbytes))
    lbm._check(L.lbm_write_field(lbm.handle, C.FIELD_U, hb["u"].ctypes.data, hb["u"].nbytes))
    lbm._check(L.lbm_write_field(lbm.handle, C.FIELD_FLAGS, hb["flags"].ctypes.data, hb["flags"].nbytes))
    lbm._check(L.lbm_initialize(lbm.handle))
    lbm._check(L.lbm_stream_collide(lbm.handle, K))
    lbm._check(L.lbm_read_field(lbm.handle, C.FIELD_RHO, out_rho.ctypes.data, out_rho.nbytes))
    lbm._check(L.lbm_read_field(lbm.handle, C.FIELD_U, out_u.ctypes.data, out_u.nbytes))
    e1.record(stream)
    e1.synchronize()
    wall = time.perf_counter() - t0
    e2e_s = max_over_ranks(dist, max(wall, e0.elapsed_time(e1) * 1e-3))
    e2e_value = world * N * K / e2e_s / 1e6
    h2d = hb["rho"].nbytes + hb["u"].nbytes + hb["flags"].nbytes
    d2h = out_rho.nbytes + out_u.nbytes
    if not np.all(np.isfinite(out_u)):
        raise RuntimeError("non-finite velocity after the end-to-end job")
    if rank != 0:
        lbm.close()
        return 0
    peak, peak_kind = measured_peaks()
    launch_s = ms * 1e-3 / K
    achieved = bpc * N / launch_s / 1e9
    traffic = traffic_per_launch()
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_run(K, time_budget_s=args.cpu_budget)
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": w["name"], "cells": N, "velocity_set": "D3Q19", "collision": "TRT", "ddf_storage": "FP16S",
                   "arithmetic": "FP32", "extensions": ["EQUILIBRIUM_BOUNDARIES"], "nu": w["nu"], "parallelism": f"replicas{world}",
                   "l2": "inputs larger than L2 (1.27 GB DDFs per step), no flush",
                   "bytes_per_cell_step": bpc},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": f"{peak_kind} hbm_gbs", "kernel": KERNEL},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d / K, "d2h_bytes_per_step": d2h / K,
                "job": f"upload rho/u/flags + initialize + {K} steps + update_fields + download rho/u"},
        "fluid_cells": fluid, "fluid_mlups": world * fluid * K / (ms_max * 1e-3) / 1e6,
        "gpu_launches": K,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line))
    lbm.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU-baseline work")
    ap.add_argument("--size", default=None, help="NXxNYxNZ instead of 512x256x256 (profiling captures of a small case)")
    args = ap.parse_args()
    if args.size:
        set_size(args.size)
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference_arm(args)
    return run_gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
