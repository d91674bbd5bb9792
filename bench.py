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
all the host cores (the reference itself needs external BLAS/LAPACK/HDF5 builds and is not
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


def build_gpu_dmrg(model, D=D_VIRT, sweeps=1, right_ops=True):
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
    scheme.set_instruction(0, D, 1e-10, sweeps, 0.0, 1e-8)
    c2g.srand(SEED)
    dmrg = c2g.DMRG(prob, scheme)
    if right_ops:
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
        fd, name = tempfile.mkstemp(prefix="c2g_clocks_", suffix=".csv")
        os.close(fd)
        self.path = Path(name)

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
    """The CPU oracle port of the same matvec on all host cores (the executor runs the
    independent output blocks of a stage on parallel threads), bounded to n_matvec
    applications after its own setup."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as ol

    threads = os.cpu_count() or 1
    ol.set_threads(threads)
    ol.srand(SEED)
    cpu = ol.OracleDMRG(model, TWO_S, N_ELEC, IRREP, [(D_VIRT, 1e-10, 1, 0.0, 1e-8)], check=False)
    for index in range(L_SITES - 2, MID, -1):
        cpu.update(index, False)
    x, _, _ = cpu.heff_apply(MID)  # joins the two-site object, compiles (untimed)
    t0 = time.perf_counter()
    for _ in range(n_matvec):
        cpu.heff_apply(MID, x)
    dt = time.perf_counter() - t0
    return {"value": n_matvec / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n_matvec} Heff matvec(s) at sites ({MID},{MID + 1}) of the same L=24 D=1000 state "
                      f"(oracle CPU executor on {threads} threads, compile excluded, as for the GPU)"}


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


def sweep_config2(model, sweeps=2, steps=20):
    """The headline system (L = 24, D = 1000) swept `sweeps` times from the random start in
    plain FP64 and in mixed precision: seconds per sweep (first and last sweep, host task
    compilation included), the energy difference, and the matvec rate at sites (11, 12) on
    the swept state (sector dimensions after truncation, larger blocks than the initial
    state), FP64 and FP32."""
    out = {"config": f"synthetic ab initio L=24 N=24 S=0 D2h D=1000, {sweeps} sweeps, Davidson rtol 1e-8"}
    for mode in ("fp64", "mixed"):
        ham, prob, scheme, d = build_gpu_dmrg(model, sweeps=1, right_ops=False)  # one sweep per Solve()
        d.set_precision(mode)
        per = []
        for _ in range(sweeps):
            d.reset_stats()
            t0 = time.perf_counter()
            e = d.Solve()
            per.append(time.perf_counter() - t0)
        st = d.stats()
        res = {"s_per_sweep": per, "energy": e, "last_sweep": {k: v for k, v in st.items() if k.startswith(("t_", "n_"))}}
        if mode == "fp64":
            for index in range(L_SITES - 2, MID, -1):
                d.update(index, False)
            r64 = d.bench_heff(MID, 3, steps, L2_FLUSH_BYTES)
            r32 = d.bench_heff(MID, 3, steps, L2_FLUSH_BYTES, precision="fp32")
            res["swept_state_matvec"] = {
                "fp64_matvec_per_s": 1e3 / r64["ms_per_matvec"], "fp64_gflops": r64["flops"] / r64["ms_per_matvec"] / 1e6,
                "fp32_matvec_per_s": 1e3 / r32["ms_per_matvec"], "fp32_gflops": r32["flops"] / r32["ms_per_matvec"] / 1e6,
                "ledger_flops_per_matvec": r64["flops"], "two_site_vector_length": d.sobject_size(MID)}
        d.close()
        out[mode] = res
    out["mixed_speedup_last_sweep"] = out["fp64"]["s_per_sweep"][-1] / out["mixed"]["s_per_sweep"][-1]
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
    sweep = sweep24 = None
    if rank == 0 and not args.no_sweep:
        sweep = sweep_seconds()
        sweep24 = sweep_config2(model)
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
            "gpu_launches": res["launches"], "sweep": sweep, "sweep_l24_d1000": sweep24, "mixed": mixed,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def extra_config3(args):
    """Precision form: synthetic ab initio L = N = 30, S = 0, D2h, D = 2000, swept in plain
    FP64 and in mixed precision (FP32 Davidson expansion with FP64 refinement, FP64
    truncation): seconds per sweep and the energy difference. --sweeps sets the number of
    sweeps (8 in the reference configuration)."""
    import chemps2_gb300 as c2g
    from chemps2_gb300.models import synthetic_ab_initio

    L = 30
    model = synthetic_ab_initio(L, GROUP, SEED)
    out = {"config": f"synthetic ab initio L=30 N=30 S=0 D2h D=2000, {args.sweeps} sweeps, Davidson rtol 1e-8"}
    if args.profile:
        # profiling mode: --sweeps FP64 sweeps, right-hand operators down to the middle, then
        # --profile matvecs at sites (14, 15) in each precision between cudaProfilerStart/Stop
        import torch

        ham = c2g.Hamiltonian(L, model.group, model.irreps)
        for i in range(L):
            for j in range(i, L):
                if model.tmat[i, j] != 0.0:
                    ham.setTmat(i, j, float(model.tmat[i, j]))
        for i, j, k, l in np.argwhere(model.vmat != 0.0):
            if i <= j and i <= k:
                ham.setVmat(int(i), int(j), int(k), int(l), float(model.vmat[i, j, k, l]))
        prob = c2g.Problem(ham, 0, L, 0)
        scheme = c2g.ConvergenceScheme(1)
        scheme.set_instruction(0, 2000, 1e-10, args.sweeps, 0.0, 1e-8)
        c2g.srand(SEED)
        d = c2g.DMRG(prob, scheme)
        d.Solve()
        mid = L // 2 - 1
        for index in range(L - 2, mid, -1):
            d.update(index, False)
        precs = ["fp64", "fp32"]
        for p in precs:
            d.bench_heff(mid, args.warmup, 0, 0, precision=p)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        for p in precs:
            d.bench_heff(mid, 0, args.profile, 0, precision=p)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        for p in precs:
            r = d.bench_heff(mid, 0, 5, L2_FLUSH_BYTES, precision=p)
            print(json.dumps({"precision": p, "ms_per_matvec": r["ms_per_matvec"], "ledger_flops": r["flops"],
                              "ledger_bytes": r["bytes"], "n": d.sobject_size(mid)}), flush=True)
        d.close()
        return
    for mode in ("fp64", "mixed"):
        ham = c2g.Hamiltonian(L, model.group, model.irreps)
        for i in range(L):
            for j in range(i, L):
                if model.tmat[i, j] != 0.0:
                    ham.setTmat(i, j, float(model.tmat[i, j]))
        for i, j, k, l in np.argwhere(model.vmat != 0.0):
            if i <= j and i <= k:
                ham.setVmat(int(i), int(j), int(k), int(l), float(model.vmat[i, j, k, l]))
        prob = c2g.Problem(ham, 0, L, 0)
        scheme = c2g.ConvergenceScheme(1)
        scheme.set_instruction(0, 2000, 1e-10, 1, 0.0, 1e-8)
        c2g.srand(SEED)
        d = c2g.DMRG(prob, scheme)
        d.set_precision(mode)
        per, stats = [], []
        for _ in range(args.sweeps):
            d.reset_stats()
            t0 = time.perf_counter()
            e = d.Solve()
            per.append(time.perf_counter() - t0)
            stats.append({k: v for k, v in d.stats().items() if k.startswith(("t_", "n_"))})
        d.close()
        out[mode] = {"s_per_sweep": per, "energy": e, "stats": stats}
    out["mixed_speedup_last_sweep"] = out["fp64"]["s_per_sweep"][-1] / out["mixed"]["s_per_sweep"][-1]
    out["mixed_speedup_total"] = sum(out["fp64"]["s_per_sweep"]) / sum(out["mixed"]["s_per_sweep"])
    out["mixed_energy_error"] = abs(out["mixed"]["energy"] - out["fp64"]["energy"])
    print(json.dumps({"extra": "precision_l30_d2000", **out}), flush=True)


def extra_hubbard(args):
    """Large sector blocks: the Hubbard chain L = N = 20, U = 4, C1, D = 512 swept --sweeps
    times, right-hand operators renormalized down to the middle, then --steps FP64 and FP32
    matvecs at sites (9, 10) (the two-pass path of large groups carries most of the work).
    With --profile n: n matvecs (--profile-precision) between cudaProfilerStart/Stop,
    nothing printed."""
    import torch

    import chemps2_gb300 as c2g
    from chemps2_gb300.models import hubbard

    L, mid = 20, 9
    m = hubbard(L, 4.0)
    ham = c2g.Hamiltonian(L, 0, m.irreps)
    for i in range(L - 1):
        ham.setTmat(i, i + 1, -1.0)
    for i in range(L):
        ham.setVmat(i, i, i, i, 4.0)
    prob = c2g.Problem(ham, 0, L, 0)
    scheme = c2g.ConvergenceScheme(1)
    scheme.set_instruction(0, 512, 1e-10, args.sweeps, 0.0, 1e-8)
    c2g.srand(7)
    d = c2g.DMRG(prob, scheme)
    t0 = time.perf_counter()
    e = d.Solve()
    solve_s = time.perf_counter() - t0
    for index in range(L - 2, mid, -1):
        d.update(index, False)
    d.bench_heff(mid, args.warmup, 0, 0)
    if args.profile:
        d.bench_heff(mid, args.warmup, 0, 0, precision=args.profile_precision)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        d.bench_heff(mid, 0, args.profile, 0, precision=args.profile_precision)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        d.close()
        return
    r64 = d.bench_heff(mid, 0, args.steps, L2_FLUSH_BYTES)
    d.bench_heff(mid, args.warmup, 0, 0, precision="fp32")
    r32 = d.bench_heff(mid, 0, args.steps, L2_FLUSH_BYTES, precision="fp32")
    d.close()
    out = {"config": f"hubbard L=20 N=20 U=4 C1 D=512, {args.sweeps} sweep(s), matvec at sites (9,10)",
           "solve_s": solve_s, "energy": e,
           "fp64": {"ms_per_matvec": r64["ms_per_matvec"], "gflops": r64["flops"] / r64["ms_per_matvec"] / 1e6,
                    "launches_per_matvec": r64["launches"] / max(args.steps, 1)},
           "fp32": {"ms_per_matvec": r32["ms_per_matvec"], "gflops": r32["flops"] / r32["ms_per_matvec"] / 1e6},
           "ledger_flops_per_matvec": r64["flops"]}
    print(json.dumps({"extra": "hubbard_l20_d512", **out}), flush=True)


def batch_objects(members, sweeps):
    import chemps2_gb300 as c2g

    objs = []
    for mb in members:
        m = mb["model"]
        ham = c2g.Hamiltonian(m.L, m.group, m.irreps)
        for i in range(m.L):
            for j in range(i, m.L):
                if m.tmat[i, j] != 0.0:
                    ham.setTmat(i, j, float(m.tmat[i, j]))
        for i, j, k, l in np.argwhere(m.vmat != 0.0):
            if i <= j and i <= k:
                ham.setVmat(int(i), int(j), int(k), int(l), float(m.vmat[i, j, k, l]))
        prob = c2g.Problem(ham, mb["two_s"], mb["n"], mb["irrep"])
        sc = c2g.ConvergenceScheme(1)
        sc.set_instruction(0, mb["D"], 1e-10, sweeps, 0.0, 1e-8)
        objs.append((ham, prob, sc))
    return objs


def extra_batch(args):
    """Batching form: the seeded set of independent problems (L in 8..20, N = L, half
    Hubbard, half synthetic ab initio, D in {64, 128, 256, 512}, FP64), --batch-count of
    them (64 in the reference configuration), each swept --sweeps times, solved
    concurrently through c2g_batch_solve (each problem on its own stream, --workers host
    threads) and one after another: aggregate Heff matvecs/s both ways, with the energies
    of the two runs compared."""
    import chemps2_gb300 as c2g
    from chemps2_gb300.models import batch_members

    members = batch_members(args.batch_count)
    out = {"config": f"{args.batch_count} problems, {args.sweeps} sweep(s) each, FP64"}
    energies = {}
    for label, workers in (("concurrent", args.workers), ("sequential", 1)):
        objs = batch_objects(members, args.sweeps)
        t0 = time.perf_counter()
        res = c2g.solve_batch([o[1] for o in objs], [o[2] for o in objs], [mb["seed"] for mb in members],
                              workers=workers)
        dt = time.perf_counter() - t0
        mv = sum(r["matvecs"] for r in res)
        out[label] = {"workers": workers, "seconds": dt, "matvecs": mv, "matvec_per_s": mv / dt,
                      "device_matvec_seconds": sum(r["stats"]["t_matvec"] for r in res),
                      "compile_seconds": sum(r["stats"]["t_compile"] for r in res)}
        energies[label] = [r["energy"] for r in res]
    out["speedup"] = out["concurrent"]["matvec_per_s"] / out["sequential"]["matvec_per_s"]
    out["max_energy_difference"] = max(abs(a - b) for a, b in zip(energies["concurrent"], energies["sequential"]))
    print(json.dumps({"extra": "batch", **out}), flush=True)


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
    ap.add_argument("--extra", choices=["config3", "batch", "hubbard"], default=None,
                    help="run one of the further configurations instead (prints its own JSON line)")
    ap.add_argument("--sweeps", type=int, default=2, help="sweeps per problem for --extra")
    ap.add_argument("--batch-count", type=int, default=64, help="problems for --extra batch")
    ap.add_argument("--workers", type=int, default=16, help="concurrent problems for --extra batch")
    ap.add_argument("--profile-precision", choices=["fp64", "fp32"], default="fp64",
                    help="arithmetic of the profiled matvecs of --extra hubbard --profile")
    ap.add_argument("--profile", type=int, default=0,
                    help="profiling mode: set up, then run this many matvecs between cudaProfilerStart/Stop")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.extra == "config3":
        extra_config3(args)
    elif args.extra == "batch":
        extra_batch(args)
    elif args.extra == "hubbard":
        extra_hubbard(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
