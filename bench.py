#!/usr/bin/env python3
"""Benchmark of the two-site DMRG hot path on GB300: Heff matvecs/s.

Workload (the configuration the headline metric is quoted on): synthetic ab initio
Hamiltonian, L = N = 24, S = 0, D2h with irreps round robin, target irrep 0, virtual
dimension D = 1000 (seeded generator chemps2_gb300/models.py, seed 1234). The DMRG object
is built as the reference builds it (random MPS, sector dimensions of
SyBookkeeper::ScaleCURdim for D = 1000, all renormalized operators), the right-hand
operators are renormalized down to the middle of the chain, and one step is one
effective-Hamiltonian matvec at sites (11, 12) in FP64: the operation the Davidson
solver repeats inside every sweep step.

  value   device matvecs/s (CUDA events on the DMRG stream, L2 overwritten between
          steps outside the timed interval)
  e2e     the same matvec through the C-ABI with host buffers (c2g_dmrg_heff_apply):
          copy of x to the device, matvec, copy of y back, wall clock
  sweep   seconds per left+right sweep of the Hubbard chain L = 16, D = 200 (the CPU
          configuration of the reference's benchmark list), after one warm-up sweep

The reference arm (--impl reference) times the CPU oracle port of the same matvec on
the host cores (the reference itself needs external BLAS/LAPACK/HDF5 builds and is not
compiled here). Multi-GPU runs are independent replicas (the path has no exchange step
on one problem): each rank runs the full workload on its own GPU.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

L_SITES, N_ELEC, TWO_S, IRREP, GROUP, D_VIRT, SEED = 24, 24, 0, 0, 7, 1000, 1234
MID = L_SITES // 2 - 1
L2_FLUSH_BYTES = 2 * 129 * 1024 * 1024
METRIC = "Heff matvecs/s & s/sweep: mixed vs FP64 GPU at ≤1e-6 Ha; CPU ref"
UNIT = "matvec/s"


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(seconds, world, device="cuda"):
    """The slowest rank's time: every rank runs the same replica workload and the job ends
    with the slowest one (no data-path collective; this is the only exchange)."""
    if world <= 1:
        return seconds
    import torch

    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, steps, seconds):
    """Whole-job units per second: `steps` units on each of `world` replicas."""
    return world * steps / seconds


def make_model():
    from chemps2_gb300.models import synthetic_ab_initio

    return synthetic_ab_initio(L_SITES, GROUP, SEED)


def build_gpu_dmrg(model, D=D_VIRT):
    import chemps2_gb300 as c2g

    L = model.L
    ham = c2g.Hamiltonian(L, model.group, model.irreps)
    for i in range(L):
        for j in range(i, L):
            if model.tmat[i, j] != 0.0:
                ham.setTmat(i, j, float(model.tmat[i, j]))
    for i, j, k, l in np.argwhere(model.vmat != 0.0):
        if i <= j and i <= k:  # one representative of each 8-fold orbit
            ham.setVmat(int(i), int(j), int(k), int(l), float(model.vmat[i, j, k, l]))
    prob = c2g.Problem(ham, TWO_S, N_ELEC, IRREP)
    scheme = c2g.ConvergenceScheme(1)
    scheme.set_instruction(0, D, 1e-10, 1, 0.0, 1e-8)
    c2g.srand(SEED)
    dmrg = c2g.DMRG(prob, scheme)
    for index in range(L - 2, MID, -1):  # right-hand operators down to the middle
        dmrg.update(index, False)
    return ham, prob, scheme, dmrg


class ClockSampler:
    """nvidia-smi samples of the SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = Path(tempfile.mkstemp(prefix="c2g_clocks_", suffix=".csv")[1])

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        self.path.unlink(missing_ok=True)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        return {}


def profiled_traffic():
    """DRAM bytes per Heff launch from the committed ncu summary (scaled to this workload)."""
    try:
        prof = json.loads((ROOT / "profiles" / "heff_team_kernel_l24_d1000.json").read_text())
        return prof.get("dram_bytes_per_matvec")
    except (OSError, ValueError):
        return None


def cpu_baseline_sample(model, n_matvec=1):
    """The CPU oracle port of the same matvec (single host thread), bounded to n_matvec
    applications after its own setup."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as ol

    ol.srand(SEED)
    cpu = ol.OracleDMRG(model, TWO_S, N_ELEC, IRREP, [(D_VIRT, 1e-10, 1, 0.0, 1e-8)], check=False)
    for index in range(L_SITES - 2, MID, -1):
        cpu.update(index, False)
    x, _, _ = cpu.heff_apply(MID)  # joins the two-site object, compiles (untimed)
    t0 = time.perf_counter()
    for _ in range(n_matvec):
        cpu.heff_apply(MID, x)
    dt = time.perf_counter() - t0
    return {"value": n_matvec / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{n_matvec} Heff matvec(s) at sites ({MID},{MID + 1}) of the same L=24 D=1000 state "
                      "(oracle CPU executor, compile excluded, as for the GPU)"}


def sweep_seconds():
    """The Hubbard chain L = 16, U = 4, D = 200 with 4 left+right sweeps (the reference's
    CPU-runnable configuration), plain FP64 and mixed precision: seconds per sweep over the
    whole run (compilation and the first sweeps from the random start included) and the
    energy difference between the two."""
    import chemps2_gb300 as c2g
    from chemps2_gb300.models import hubbard

    L = 16
    m = hubbard(L, 4.0)
    out = {"config": "hubbard L=16 N=16 U=4 D=200, 4 sweeps, Davidson rtol 1e-8"}
    for mode in ("fp64", "mixed"):
        ham = c2g.Hamiltonian(L, 0, m.irreps)
        for i in range(L - 1):
            ham.setTmat(i, i + 1, -1.0)
        for i in range(L):
            ham.setVmat(i, i, i, i, 4.0)
        prob = c2g.Problem(ham, 0, L, 0)
        scheme = c2g.ConvergenceScheme(1)
        scheme.set_instruction(0, 200, 1e-14, 4, 0.0, 1e-8)
        c2g.srand(1)
        d = c2g.DMRG(prob, scheme)
        d.set_precision(mode)
        t0 = time.perf_counter()
        e = d.Solve()
        dt = time.perf_counter() - t0
        st = d.stats()
        d.close()
        out[mode] = {"s_per_sweep": dt / 4, "energy": e, "matvecs": st["n_matvec"],
                     "fp32_matvecs": st["n_matvec_fp32"]}
    out["s_per_sweep"] = out["fp64"]["s_per_sweep"]
    out["mixed_speedup"] = out["fp64"]["s_per_sweep"] / out["mixed"]["s_per_sweep"]
    out["mixed_energy_error"] = abs(out["mixed"]["energy"] - out["fp64"]["energy"])
    return out


def run_ours(args):
    import torch

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)

    model = make_model()
    t_setup = time.perf_counter()
    ham, prob, scheme, dmrg = build_gpu_dmrg(model)
    setup_s = time.perf_counter() - t_setup
    n = dmrg.sobject_size(MID)
    # warm-up (untimed): compile + W applications
    dmrg.bench_heff(MID, args.warmup, 0, 0)
    if args.profile:
        # profiling mode: one launch sequence of one matvec between cudaProfilerStart/Stop
        # (for ncu --profile-from-start off); prints nothing.
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        dmrg.bench_heff(MID, 0, args.profile, 0)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        dmrg.close()
        return
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        res = dmrg.bench_heff(MID, 0, args.steps, L2_FLUSH_BYTES)
    torch.cuda.synchronize()
    ms = res["ms_per_matvec"]
    total_s = ms * args.steps / 1e3
    # the FP32-arithmetic matvec of the mixed-precision Davidson, same flush discipline
    dmrg.bench_heff(MID, args.warmup, 0, 0, precision="fp32")
    res32 = dmrg.bench_heff(MID, 0, args.steps, L2_FLUSH_BYTES, precision="fp32")
    mixed = {"matvec_per_s": 1e3 / res32["ms_per_matvec"], "ms_per_matvec": res32["ms_per_matvec"],
             "speedup_vs_fp64": ms / res32["ms_per_matvec"],
             "arithmetic": "FP32 operand copies, products and per-slot sums; FP64 slot reduction and output"}
    total_s = max_over_ranks(total_s, world)
    if world > 1:
        torch.distributed.barrier()
    value = replica_throughput(world, args.steps, total_s)
    # end to end through the C-ABI with host buffers
    rng = np.random.default_rng(0)
    x = rng.standard_normal(n)
    dmrg.heff_apply(MID, x)  # warm
    t0 = time.perf_counter()
    for _ in range(args.steps):
        dmrg.heff_apply(MID, x)
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, world)
    e2e = {"value": replica_throughput(world, args.steps, e2e_s), "unit": UNIT, "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n}
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    achieved = res["bytes"] / (ms * 1e-3) / 1e9
    # The kernel is bound by the FP64 pipe, not by HBM: the compute roofline sits beside the
    # HBM one. FP64 peak = ncu's device peak of 608 FP64 flops per cycle (2 DFMA lanes per SM
    # and cycle) at the maximum SM clock; FP32 peak likewise 38912 flops per cycle.
    sm_hz = float(peaks.get("sm_max_mhz", 2070.0)) * 1e6
    fp64_peak = 608 * sm_hz / 1e9
    fp32_peak = 38912 * sm_hz / 1e9
    gflops = res["flops"] / (ms * 1e-3) / 1e9
    gflops32 = res32["flops"] / (res32["ms_per_matvec"] * 1e-3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm if hbm else 6800.0,
                "unit": "GB/s", "frac": achieved / (hbm if hbm else 6800.0), "traffic": profiled_traffic(),
                "peak_source": "measured" if hbm else "fallback",
                "kernel": "sandwich_warp_kernel<double, R> (team block sandwich, one launch per row class)",
                "ledger_bytes_per_matvec": res["bytes"], "ledger_flops_per_matvec": res["flops"],
                "compute": {"pipe": "fp64", "achieved_gflops": gflops, "peak_gflops": fp64_peak,
                            "frac": gflops / fp64_peak,
                            "peak_source": "ncu device peak 608 FP64 flop/cycle x max SM clock"},
                "compute_fp32_variant": {"pipe": "fp32", "achieved_gflops": gflops32, "peak_gflops": fp32_peak,
                                         "frac": gflops32 / fp32_peak}}
    dmrg.close()
    sweep = None
    if rank == 0 and not args.no_sweep:
        sweep = sweep_seconds()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline_sample(model, n_matvec=1)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded ab initio generator, seed 1234)",
            "config": {"workload": "synthetic ab initio L=24 N=24 S=0 D2h D=1000, Heff matvec at sites (11,12), "
                                   "initial SyBookkeeper dimensions", "L": L_SITES, "N": N_ELEC, "two_s": TWO_S,
                       "group": "D2h", "D": D_VIRT, "two_site_vector_length": n, "l2": "flushed between steps",
                       "parallelism": f"replicas x{world}", "setup_s": setup_s},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk.summary(),
            "gpu_launches": res["launches"], "sweep": sweep, "mixed": mixed,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    model = make_model()
    steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    cb = cpu_baseline_sample(model, n_matvec=steps)
    wall = time.perf_counter() - t0
    line = {
        "impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 / cb["value"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded ab initio generator, seed 1234)",
        "config": {"workload": "synthetic ab initio L=24 N=24 S=0 D2h D=1000, Heff matvec at sites (11,12), "
                               "initial SyBookkeeper dimensions", "setup_and_sample_s": wall},
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU oracle port of the reference's Heff (the reference needs BLAS/LAPACK/HDF5 builds absent here)",
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-sweep", action="store_true", help="skip the sweep timing")
    ap.add_argument("--profile", type=int, default=0,
                    help="profiling mode: set up, then run this many matvecs between cudaProfilerStart/Stop")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
