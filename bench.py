#!/usr/bin/env python3
"""Benchmark of the two-site DMRG hot path on GB300: Heff matvecs/s and s/sweep, mixed
precision against FP64 on the GPU, with the CPU baseline alongside.

Workload (the configuration the headline metric is quoted on): seeded synthetic ab initio
Hamiltonian, L = N = 30, S = 0, D2h with irreps round robin, target irrep 0, virtual
dimension D = 2000 (generator chemps2_gb300/models.py, seed 1234; no molecule data ships
with the reference's benchmarks, so seeded integrals of the configuration's distribution
stand in). Two DMRG runs from the same random start (srand(1234)), each swept --sweeps
times (left + right sweeps, Davidson rtol 1e-8, noise 0):

  fp64      plain FP64 matvecs (the reference's arithmetic)
  mixed_tc  the Davidson solver expands with reduced-precision matvecs whose large
            blocks run on the tensor cores (tcgen05, split-BF16 three-term products,
            FP32 accumulation; the rest FP32), then refines with FP64 products to rtol

Then, on the FP64 run's swept state with the right-hand operators renormalized down to
the middle, one step = one Heff matvec at sites (14, 15):

  value     mixed-form (tensor-core) matvecs/s, device time (CUDA events on the DMRG's
            stream; a 258 MiB buffer is overwritten between steps, outside the timed
            interval, so the operators come from HBM)
  e2e       the same matvec through the C-ABI with host buffers
            (c2g_dmrg_heff_apply_precision): x copied in, matvec, y copied out, wall clock
  fp64 / fp32  the same state's FP64 and all-FP32 matvec rates
  sweeps    seconds per sweep of both runs, their energy difference and the time split
            (matvecs, task compilation, upload, truncation, operator updates)

The reference arm (--impl reference) and `cpu_baseline` time the CPU oracle's port of the
same matvec on all host cores, on a state with the swept state's sector dimensions (the
reference itself needs external BLAS/LAPACK/HDF5 builds and is not compiled here).
Multi-GPU runs are independent replicas (one problem has no exchange step on one GPU):
each rank runs the full workload on its own GPU.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

L_SITES, N_ELEC, TWO_S, IRREP, GROUP, D_VIRT, SEED = 30, 30, 0, 0, 7, 2000, 1234
MID = L_SITES // 2 - 1
L2_FLUSH_BYTES = 2 * 129 * 1024 * 1024
METRIC = "Heff matvecs/s & s/sweep: mixed vs FP64 GPU at ≤1e-6 Ha; CPU ref"
UNIT = "matvec/s"
WORKLOAD = (f"synthetic ab initio L={L_SITES} N={N_ELEC} S=0 D2h D={D_VIRT}: Heff matvec at sites ({MID},{MID + 1}) "
            f"of the state after the FP64 sweeps, mixed (tensor-core) form; FP64 and mixed sweeps")
# Sector dimensions of every boundary of the L = 30 D = 2000 state after the two FP64
# sweeps of the GPU run (written by `bench.py --dump-dims`): the CPU baseline builds a
# state with exactly these dimensions, so that its matvec has the same shape and ledger
# work as the GPU's.
DIMS_FIXTURE = ROOT / "oracle" / "bench_l30_d2000_swept_dims.json"


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


def make_model(L=L_SITES):
    from chemps2_gb300.models import synthetic_ab_initio

    return synthetic_ab_initio(L, GROUP, SEED)


def build_gpu_dmrg(model, D=D_VIRT, sweeps=1, seed=SEED):
    """The DMRG objects of `model` (N = L, S = 0, target irrep 0) with one instruction of
    `sweeps` sweeps at D, after srand(seed)."""
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
    prob = c2g.Problem(ham, TWO_S, L, IRREP)
    scheme = c2g.ConvergenceScheme(1)
    scheme.set_instruction(0, D, 1e-10, sweeps, 0.0, 1e-8)
    c2g.srand(seed)
    dmrg = c2g.DMRG(prob, scheme)
    return ham, prob, scheme, dmrg


def host_cpu():
    model = platform.processor() or platform.machine()
    try:
        for line in subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return model


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
    """DRAM bytes per mixed-form matvec from the committed ncu summary (None when absent)."""
    try:
        prof = json.loads((ROOT / "profiles" / "heff_mixed_tc_l30_d2000.json").read_text())
        return prof.get("dram_bytes_per_matvec")
    except (OSError, ValueError):
        return None


def swept_dims():
    try:
        return json.loads(DIMS_FIXTURE.read_text())["rows"]
    except (OSError, ValueError, KeyError):
        return None


def state_dims(dmrg, L=L_SITES):
    return [[b, int(r[0]), int(r[1]), int(r[2]), int(r[4])] for b in range(L + 1) for r in dmrg.sectors(b)
            if r[4] > 0]


def cpu_baseline_sample(n_matvec=3, n_warmup=1):
    """The CPU oracle's port of the same matvec on all host cores (its executor runs the
    independent output blocks of a stage on parallel threads): a state of the L = 30
    D = 2000 chain with the sector dimensions of the GPU run's swept state (random tensors:
    the matvec's work depends on the dimensions only), left operators up to the middle,
    right operators down to it, then n_matvec timed matvecs at sites (14, 15) after
    n_warmup untimed ones (the first of which joins the two-site object and compiles the
    program). Without the dimensions file, the initial (scaled) dimensions of D = 2000."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as ol

    threads = os.cpu_count() or 1
    ol.set_threads(threads)
    ol.srand(SEED)
    model = make_model()
    rows = swept_dims()
    sched = [(D_VIRT, 1e-10, 1, 0.0, 1e-8)]
    t0 = time.perf_counter()
    if rows is not None:
        cpu = ol.OracleDMRG(model, TWO_S, N_ELEC, IRREP, sched, check=False, dims=rows, left_upto=MID)
        state = "the sector dimensions of the GPU run's swept state"
    else:
        cpu = ol.OracleDMRG(model, TWO_S, N_ELEC, IRREP, sched, check=False)
        state = "the initial sector dimensions"
    for index in range(L_SITES - 2, MID, -1):
        cpu.update(index, False)
    x, _, _ = cpu.heff_apply(MID)  # joins the two-site object, compiles, first matvec (untimed)
    for _ in range(max(n_warmup, 1) - 1):
        cpu.heff_apply(MID, x)
    setup = time.perf_counter() - t0
    f0 = cpu.stats()["flops"]
    t0 = time.perf_counter()
    for _ in range(n_matvec):
        cpu.heff_apply(MID, x)
    dt = time.perf_counter() - t0
    flops = (cpu.stats()["flops"] - f0) / n_matvec
    return {"value": n_matvec / dt, "unit": UNIT, "cores": threads, "kind": "port", "cpu": host_cpu(),
            "flops_per_matvec": flops, "two_site_vector_length": int(x.size), "setup_s": setup,
            "sample": f"{n_matvec} FP64 Heff matvecs ({max(n_warmup, 1)} untimed before them) at sites "
                      f"({MID},{MID + 1}) of L={L_SITES} D={D_VIRT} with "
                      f"{state} (oracle CPU executor, {threads} threads; compile and setup excluded, as for the "
                      f"GPU)"}


def run_sweeps(model, mode, sweeps, D=D_VIRT, seed=SEED):
    """`sweeps` left+right sweeps from the seeded random start in `mode`; returns the DMRG
    objects and the per-sweep record."""
    objs = build_gpu_dmrg(model, D=D, sweeps=1, seed=seed)
    d = objs[3]
    d.set_precision(mode)
    per, stats = [], []
    e = None
    for _ in range(sweeps):
        d.reset_stats()
        t0 = time.perf_counter()
        e = d.Solve()
        per.append(time.perf_counter() - t0)
        stats.append({k: (round(v, 4) if isinstance(v, float) else v) for k, v in d.stats().items()
                      if k.startswith(("t_", "n_"))})
    return objs, {"s_per_sweep": per, "energy": e, "stats": stats}


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
    sweeps = {}
    keep = None
    for mode in ("mixed_tc", "fp64"):
        objs, rec = run_sweeps(model, mode, args.sweeps)
        sweeps[mode] = rec
        if mode == "fp64":
            keep = objs
        else:
            objs[3].close()
    dmrg = keep[3]
    dims = state_dims(dmrg)
    if args.dump_dims:
        Path(args.dump_dims).write_text(json.dumps({
            "about": f"sector dimensions (boundary, N, 2S, I, dim) of the synthetic ab initio L={L_SITES} D2h "
                     f"D={D_VIRT} state after {args.sweeps} FP64 sweeps from srand({SEED}); written by "
                     f"bench.py --dump-dims",
            "rows": dims}) + "\n")
    fixture = swept_dims()
    dims_match = (fixture == dims) if fixture is not None else None
    for index in range(L_SITES - 2, MID, -1):  # right-hand operators down to the middle
        dmrg.update(index, False)
    setup_s = time.perf_counter() - t_setup
    n = dmrg.sobject_size(MID)
    for p in ("tc", "fp64", "fp32"):  # compile + warm-up (untimed)
        dmrg.bench_heff(MID, args.warmup, 0, 0, precision=p)
    if args.profile:
        # profiling mode: --profile matvecs of each precision between cudaProfilerStart/Stop
        # (for ncu --profile-from-start off); prints nothing.
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        for p in ("tc", "fp64", "fp32"):
            dmrg.bench_heff(MID, 0, args.profile, 0, precision=p)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        dmrg.close()
        return
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        res = dmrg.bench_heff(MID, 0, args.steps, L2_FLUSH_BYTES, precision="tc")
    torch.cuda.synchronize()
    ms = res["ms_per_matvec"]
    total_s = max_over_ranks(ms * args.steps / 1e3, world)
    if world > 1:
        torch.distributed.barrier()
    value = replica_throughput(world, args.steps, total_s)
    r64 = dmrg.bench_heff(MID, 0, args.steps, L2_FLUSH_BYTES, precision="fp64")
    r32 = dmrg.bench_heff(MID, 0, args.steps, L2_FLUSH_BYTES, precision="fp32")
    # end to end through the C-ABI with host buffers, same arithmetic as `value`
    rng = np.random.default_rng(0)
    x = rng.standard_normal(n)
    dmrg.heff_apply_precision(MID, x, "tc")  # warm
    t0 = time.perf_counter()
    for _ in range(args.steps):
        dmrg.heff_apply_precision(MID, x, "tc")
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = {"value": replica_throughput(world, args.steps, e2e_s), "unit": UNIT, "h2d_bytes_per_step": 8 * n,
           "d2h_bytes_per_step": 8 * n}
    y64 = dmrg.heff_apply_precision(MID, x, "fp64")
    ytc = dmrg.heff_apply_precision(MID, x, "tc")
    tc_rel_err = float(np.linalg.norm(ytc - y64) / np.linalg.norm(y64))
    dmrg.close()

    peaks = measured_peaks()
    sm_hz = float(peaks.get("sm_max_mhz", 2070.0)) * 1e6
    bf16_peak = peaks.get("bf16_tflops")
    fp64_peak = 608 * sm_hz / 1e12  # ncu device attribute: 608 FP64 flop/cycle on this GPU
    fp32_peak = 38912 * sm_hz / 1e12
    tflops = res["flops"] / (ms * 1e-3) / 1e12
    t64 = r64["flops"] / (r64["ms_per_matvec"] * 1e-3) / 1e12
    t32 = r32["flops"] / (r32["ms_per_matvec"] * 1e-3) / 1e12
    hbm = peaks.get("hbm_gbs") or 6800.0
    peak = bf16_peak or 1900.0
    roofline = {"bound": "tensor", "achieved": tflops, "peak": peak, "unit": "TFLOP/s", "frac": tflops / peak,
                "traffic": profiled_traffic(),
                "peak_source": "measured bf16 dense (burst)" if bf16_peak else "fallback bf16 dense (1.9 PFLOP/s)",
                "kernel": "mixed-form Heff matvec (tcgen05 sum_tc/inter_tc kernels for the large groups, FP32 team "
                          "kernel for the rest); achieved = ledger flops of one matvec / its CUDA-event time",
                "ledger_flops_per_matvec": res["flops"], "ledger_bytes_per_matvec": res["bytes"],
                "hbm": {"achieved_gbs": res["bytes"] / (ms * 1e-3) / 1e9, "peak_gbs": hbm},
                "fp64_form": {"pipe": "fp64", "achieved_tflops": t64, "peak_tflops": fp64_peak,
                              "frac": t64 / fp64_peak, "peak_source": "608 FP64 flop/cycle x max SM clock"},
                "fp32_form": {"pipe": "fp32", "achieved_tflops": t32, "peak_tflops": fp32_peak,
                              "frac": t32 / fp32_peak}}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline_sample(n_matvec=3)
    if rank == 0:
        f64, mx = sweeps["fp64"], sweeps["mixed_tc"]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16x3",
            "arithmetic": "split-BF16 three-term tensor-core products with FP32 accumulation for the large groups, "
                          "FP32 elsewhere, FP64 output; FP64 refinement inside the solver",
            "data": "synthetic (seeded ab initio generator, seed 1234)",
            "config": {"workload": WORKLOAD, "L": L_SITES, "N": N_ELEC, "two_s": TWO_S, "group": "D2h",
                       "D": D_VIRT, "sweeps": args.sweeps, "two_site_vector_length": n,
                       "state_dims_equal_cpu_baseline_state": dims_match,
                       "l2": "flushed between steps (258 MiB overwrite outside the timed interval)",
                       "parallelism": f"replicas x{world}", "setup_s": setup_s},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk.summary(),
            "gpu_launches": res["launches"],
            "fp64": {"matvec_per_s": 1e3 / r64["ms_per_matvec"], "ms_per_matvec": r64["ms_per_matvec"]},
            "fp32": {"matvec_per_s": 1e3 / r32["ms_per_matvec"], "ms_per_matvec": r32["ms_per_matvec"]},
            "mixed_matvec_speedup_vs_fp64": r64["ms_per_matvec"] / ms,
            "mixed_matvec_rel_error": tc_rel_err,
            "sweeps": {"fp64": f64, "mixed_tc": mx,
                       "mixed_speedup_last_sweep": f64["s_per_sweep"][-1] / mx["s_per_sweep"][-1],
                       "mixed_speedup_total": sum(f64["s_per_sweep"]) / sum(mx["s_per_sweep"]),
                       "mixed_energy_error": abs(mx["energy"] - f64["energy"])},
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def cpu_sweeps(model, sweeps, D, seed):
    """The CPU oracle's sweeps (its port of the reference's Solve) from the same seeded
    start, one Solve per sweep, on all host cores: seconds per sweep and the energy."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as ol

    threads = os.cpu_count() or 1
    ol.set_threads(threads)
    ol.srand(seed)
    cpu = ol.OracleDMRG(model, TWO_S, model.L, IRREP, [(D, 1e-10, 1, 0.0, 1e-8)], check=False)
    per, e = [], None
    for _ in range(sweeps):
        t0 = time.perf_counter()
        e = cpu.solve()
        per.append(time.perf_counter() - t0)
    return {"s_per_sweep": per, "energy": e, "threads": threads, "cpu": host_cpu(), "kind": "port"}


def extra_sweeps(args, label, model, D, seed=SEED, cpu=False):
    """Sweeps of another configuration in FP64 and in the mixed tensor-core form; with cpu,
    also the CPU oracle's sweeps from the same start."""
    out = {"config": f"{label}, {args.sweeps} sweeps, Davidson rtol 1e-8"}
    for mode in ("fp64", "mixed_tc"):
        objs, rec = run_sweeps(model, mode, args.sweeps, D=D, seed=seed)
        objs[3].close()
        out[mode] = rec
    out["mixed_speedup_last_sweep"] = out["fp64"]["s_per_sweep"][-1] / out["mixed_tc"]["s_per_sweep"][-1]
    out["mixed_energy_error"] = abs(out["mixed_tc"]["energy"] - out["fp64"]["energy"])
    if cpu:
        out["cpu_oracle"] = cpu_sweeps(model, args.sweeps, D, seed)
        out["fp64_speedup_vs_cpu_last_sweep"] = out["cpu_oracle"]["s_per_sweep"][-1] / out["fp64"]["s_per_sweep"][-1]
        out["fp64_energy_minus_cpu"] = out["fp64"]["energy"] - out["cpu_oracle"]["energy"]
    print(json.dumps({"extra": label, **out}), flush=True)


def extra_config5(args):
    """The large configuration: synthetic ab initio L = N = 40, S = 0, C2v (irreps round
    robin), mixed tensor-core form with every operator resident in HBM.

    First the same-D comparison at the reduced D = --reduced-d: an FP64 and a mixed run of
    --sweeps sweeps each from the same seeded start, each followed by the 2-RDM
    (calc2DMandCorrelations): energies, the 2-RDM identities (trace = N(N-1), energy of the
    2-RDM = energy of the MPS) and the Frobenius norm of the difference of the two 2-RDMs.
    Then D = 4000 in the mixed form for --large-sweeps sweeps: seconds per sweep with the
    step timers, the energy, device memory in use (the 2-RDM at D = 4000 only with
    --large-2rdm)."""
    import chemps2_gb300 as c2g
    from chemps2_gb300.models import synthetic_ab_initio

    L = 40
    model = synthetic_ab_initio(L, 5, SEED)
    out = {"config": f"synthetic ab initio L=40 N=40 S=0 C2v; FP64 and mixed at D={args.reduced_d}, "
                     f"{args.sweeps} sweep(s) each, then the 2-RDM; mixed at D=4000, {args.large_sweeps} sweep(s)"}
    rdm = {}
    for mode in (("fp64", "mixed_tc") if args.reduced_d > 0 else ()):
        objs, rec = run_sweeps(model, mode, args.sweeps, D=args.reduced_d)
        d = objs[3]
        t0 = time.perf_counter()
        d.calc2DMandCorrelations()
        t2 = time.perf_counter() - t0
        tdm = d.get2DM()
        rdm[mode] = (np.array(tdm.A), np.array(tdm.B))
        out[f"reduced_d_{mode}"] = {"s_per_sweep": rec["s_per_sweep"], "energy": rec["energy"], "stats": rec["stats"],
                                    "two_rdm_s": t2, "two_rdm_trace": tdm.trace(),
                                    "two_rdm_trace_expected": L * (L - 1), "two_rdm_energy": tdm.energy()}
        d.close()
    if args.reduced_d > 0:
        out["reduced_d_two_rdm_frobenius_diff"] = {
            "A": float(np.linalg.norm(rdm["mixed_tc"][0] - rdm["fp64"][0])),
            "B": float(np.linalg.norm(rdm["mixed_tc"][1] - rdm["fp64"][1])),
            "A_norm": float(np.linalg.norm(rdm["fp64"][0])), "B_norm": float(np.linalg.norm(rdm["fp64"][1]))}
        out["reduced_d_energy_diff"] = abs(out["reduced_d_mixed_tc"]["energy"] - out["reduced_d_fp64"]["energy"])
        print(json.dumps({"extra": "config5_reduced", **out}), flush=True)
    if args.large_sweeps <= 0:
        return
    free0, _ = c2g.device_memory_info()
    objs, rec = run_sweeps(model, "mixed_tc", args.large_sweeps, D=4000)
    d = objs[3]
    free1, used1 = c2g.device_memory_info()
    big = {"D": 4000, "s_per_sweep": rec["s_per_sweep"], "energy": rec["energy"], "stats": rec["stats"],
           "device_bytes_held_after_sweeps": free0 - free1, "pool_bytes_in_use": used1}
    if args.large_2rdm:
        t0 = time.perf_counter()
        d.calc2DMandCorrelations()
        tdm = d.get2DM()
        big.update({"two_rdm_s": time.perf_counter() - t0, "two_rdm_trace": tdm.trace(),
                    "two_rdm_trace_expected": L * (L - 1), "two_rdm_energy": tdm.energy()})
    d.close()
    print(json.dumps({"extra": "config5_large", **big}), flush=True)


def extra_hubbard(args):
    """Large sector blocks: the Hubbard chain L = N = 20, U = 4, C1, D = 512 swept --sweeps
    times, right-hand operators renormalized down to the middle, then --steps FP64, FP32 and
    tensor-core matvecs at sites (9, 10) (the two-pass path of large groups carries most of the work).
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
    d.bench_heff(mid, args.warmup, 0, 0, precision="tc")
    rtc = d.bench_heff(mid, 0, args.steps, L2_FLUSH_BYTES, precision="tc")
    d.close()
    out = {"config": f"hubbard L=20 N=20 U=4 C1 D=512, {args.sweeps} sweep(s), matvec at sites (9,10)",
           "solve_s": solve_s, "energy": e,
           "fp64": {"ms_per_matvec": r64["ms_per_matvec"], "gflops": r64["flops"] / r64["ms_per_matvec"] / 1e6,
                    "launches_per_matvec": r64["launches"] / max(args.steps, 1)},
           "fp32": {"ms_per_matvec": r32["ms_per_matvec"], "gflops": r32["flops"] / r32["ms_per_matvec"] / 1e6},
           "tc": {"ms_per_matvec": rtc["ms_per_matvec"], "gflops": rtc["flops"] / rtc["ms_per_matvec"] / 1e6},
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
    # the same K timed and W untimed steps as this script's own arm: on the 16 host cores
    # of a GB300 machine one step is about 1.8 s, so the default K = 20, W = 3 take under a
    # minute
    steps = max(1, args.steps)
    t0 = time.perf_counter()
    cb = cpu_baseline_sample(n_matvec=steps, n_warmup=max(1, args.warmup))
    wall = time.perf_counter() - t0
    line = {
        "impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 / cb["value"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded ab initio generator, seed 1234)",
        "config": {"workload": WORKLOAD, "sample": cb["sample"], "setup_and_sample_s": wall},
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU oracle port of the reference's Heff (the reference needs BLAS/LAPACK/HDF5 builds absent here)",
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[1])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--extra", choices=["config1", "config2", "config5", "batch", "hubbard"], default=None,
                    help="run one of the further configurations instead (prints its own JSON line)")
    ap.add_argument("--sweeps", type=int, default=2, help="sweeps of each run")
    ap.add_argument("--batch-count", type=int, default=64, help="problems for --extra batch")
    ap.add_argument("--workers", type=int, default=16, help="concurrent problems for --extra batch")
    ap.add_argument("--profile-precision", choices=["fp64", "fp32", "tc"], default="fp64",
                    help="arithmetic of the profiled matvecs of --extra hubbard --profile")
    ap.add_argument("--reduced-d", type=int, default=1000,
                    help="D of the FP64 2-RDM check of --extra config5 (0: skip it)")
    ap.add_argument("--large-sweeps", type=int, default=1, help="sweeps at D=4000 of --extra config5")
    ap.add_argument("--large-2rdm", action="store_true", help="also the 2-RDM at D=4000 in --extra config5")
    ap.add_argument("--dump-dims", default=None,
                    help="write the sector dimensions of the swept FP64 state to this JSON file")
    ap.add_argument("--profile", type=int, default=0,
                    help="profiling mode: set up, then run this many matvecs between cudaProfilerStart/Stop")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.extra == "config1":
        from chemps2_gb300.models import hubbard

        extra_sweeps(args, "hubbard L=16 N=16 U=4 C1 D=200", hubbard(16, 4.0), 200, seed=1, cpu=True)
    elif args.extra == "config2":
        extra_sweeps(args, "synthetic ab initio L=24 N=24 S=0 D2h D=1000", make_model(24), 1000)
    elif args.extra == "config5":
        extra_config5(args)
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
