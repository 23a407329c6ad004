"""Benchmark: RPA correlation energy of a synthetic cell on one GB300 (or N replicas, or with
--sharded one E_c split over N ranks by tau and q slices).

One step = one librpa_get_rpa_correlation_energy evaluation of the workload
(grids, G(R, +-tau) build, chi0 contraction, FT/CT, Pi / log-det / trace).

  value : seconds per E_c with the staged inputs already resident in HBM
          (handler cache reused; no host->device copy inside the timed region)
  e2e   : the same call with host buffers: every step re-stages the inputs
          host->device inside the timed region and reads the energies back
  roofline : dominant kernel (chi0 contraction), FLOPs per launch / CUDA-event time
  cpu_baseline : the oracle port (numpy + OpenBLAS, all host cores) on a bounded
          sample of the same workload, scaled to seconds per E_c

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                       [--workload fcc16_k333] [--precision bf16x3|fp32|fp64] [--fp64-check auto|on|off]
                       [--sharded]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

MEV_PER_ATOM_HA = 3.674932e-6  # 0.1 meV in Hartree
PREC = {"bf16x3": 1, "fp32": 2, "fp64": 0}


# DRAM bytes (read + write) of one per-(tau, spin) chi0 contraction launch set, from one ncu capture
# per kernel on the same workload; None where no capture exists.
PROFILED_TRAFFIC = {
    "fcc16_k333": {"bytes": 18.4119e9 + 0.0625e9 + 5.2037e9 + 0.3735e9,
                   "source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of k_t1_tc (tau_1) and the X "
                             "k_tc_gemm (tau_0); k_t2 (1.4% of time) not captured"},
}

def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.lines:
            return None
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        return ws, rank, local, dist
    return 1, 0, 0, None


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _max_over_ranks(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _opts(L, s):
    return L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                     minimax_emin=s.minimax_emin, minimax_emax=s.minimax_emax)


def _config(s):
    """The workload descriptor both arms print (identical by construction)."""
    n_sup = s.n_kpts * s.n_ao  # BvK cells = k points
    c_bytes = 8.0 * sum(a * b for a, b in zip(s.nao, s.nabf)) * n_sup
    l2 = (f"inputs larger than L2: RI matrix {c_bytes / 1e6:.0f} MB > 129 MB" if c_bytes > 129e6
          else f"RI matrix {c_bytes / 1e6:.1f} MB fits L2")
    return {"workload": s.name, "n_atoms": s.n_atoms, "n_kpts": s.n_kpts, "n_ao": s.n_ao,
            "n_abf": int(sum(s.nabf)), "nfreq": s.nfreq, "l2": l2}


def _cpu_path(s):
    """The host-core RPA path (oracle port, FP64, OpenMP + OpenBLAS) on the workload's inputs."""
    from oracle.cpu_path import CpuPath
    from oracle.rpa_oracle import Options as OO
    from librpa_gb300.synthetic import to_oracle_input
    return CpuPath(to_oracle_input(s), OO(nfreq=s.nfreq, minimax_emin=s.minimax_emin, minimax_emax=s.minimax_emax))


def cpu_sample(s):
    """CPU baseline on a bounded sample: one complete tau slice (G, X GEMMs, chi0 of every upper
    atom pair and cell, FT to every q) and the whole E_c stage (every (q, omega) LU), timed on
    all host cores; scaled to one E_c by the tau count.  Returns (seconds per E_c, description)."""
    cp = _cpu_path(s)
    t0 = time.perf_counter()
    cp.tau_slice(0)
    t_tau = time.perf_counter() - t0
    t0 = time.perf_counter()
    cp.correlation_energy()
    t_ec = time.perf_counter() - t0
    nt = len(cp.grid["tau"])
    desc = (f"oracle port (FP64; OpenMP chi0 and LU kernels, OpenBLAS GEMMs) on {os.cpu_count()} host threads: "
            f"tau slice 0 of {nt} measured {t_tau:.2f} s, the whole E_c stage ({cp.nq} q x "
            f"{len(cp.grid['omega'])} omega LU terms) measured {t_ec:.2f} s; value = {nt} x tau slice + E_c")
    return nt * t_tau + t_ec, desc


def run_reference(args, s, ws, rank, dist):
    """The reference CPU path (oracle port, the reference itself cannot be built here) on all host
    cores.  One E_c is n_tau + 1 stages: the tau slices, then the E_c stage.  Step k runs stage
    k mod (n_tau + 1) of successive passes (a new pass starts from zero at stage 0); the first
    `warmup` steps are not timed.  value = the sum over the stages of each stage's mean timed
    duration: the measured wall time of one whole E_c when every stage was timed at least once
    (steps >= n_tau + 1), which value_complete records."""
    if rank != 0:
        return
    cp = _cpu_path(s)
    nt = len(cp.grid["tau"])
    nstage = nt + 1
    times = {k: [] for k in range(nstage)}
    ec = None
    for k in range(args.warmup + args.steps):
        st = k % nstage
        if st == 0:
            cp.chi0q_tau[:] = 0.0
        t0 = time.perf_counter()
        if st < nt:
            cp.tau_slice(st)
        else:
            ec, _ = cp.correlation_energy()
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times[st].append(dt)
    timed = {k: statistics.mean(v) for k, v in times.items() if v}
    complete = len(timed) == nstage
    tau_mean = statistics.mean([v for k, v in timed.items() if k < nt]) if any(k < nt for k in timed) else None
    value = sum(timed.values())
    missing = [k for k in range(nstage) if k not in timed]
    est = {}
    if not complete:
        # not every stage ran in the timed region: the value is incomplete; an estimate that
        # fills the missing tau slices with the mean timed slice goes in its own field
        est = {"value_estimated": value + sum(tau_mean or 0.0 for k in missing if k < nt),
               "estimated_stages": missing}
    total_steps = args.steps
    line = {"impl": "reference", "metric": "rpa_ec_wall_time", "value": value, "unit": "s", "n_gpus": ws,
            "steps": total_steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(sum(v) for v in times.values()) / max(total_steps, 1),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "precision": "fp64", "parallelism": f"host cores x{os.cpu_count()}",
            "config": _config(s), "value_complete": complete, **est,
            "stage_s": {("tau_%d" % k if k < nt else "ec"): round(v, 4) for k, v in timed.items()},
            "ec": None if ec is None else ec.real,
            "cpu_baseline": {"value": value, "unit": "s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"every stage of the E_c path: {nt} tau slices (G, X GEMMs, chi0 of all "
                                       f"upper atom pairs and cells, FT) and the E_c stage; step k = stage "
                                       f"k mod {nstage}; oracle port (FP64, OpenMP chi0/LU kernels, OpenBLAS)"},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gb300(args, s, ws, rank, local, dist):
    import librpa_gb300 as L
    from librpa_gb300.build import build
    if rank == 0:
        build()
    _barrier(dist)
    lib = L.load_library()
    if lib.librpa_gb300_device_count() == 0:
        raise SystemExit("no CUDA device")
    import torch
    torch.cuda.set_device(local)
    prec = PREC[args.precision]
    opts = _opts(L, s)
    h = L.Handler()
    L.load_system(h, s)
    nq = L.n_ibz(s)

    def step(reuse):
        """One E_c through the public API: one call, or with --sharded this rank's tau slice
        (stage CHI0), the q-keyed reduce-scatter and its q slice's E_c (stage EC).  Returns
        (E_c, the call's counters; the two stages' summed when sharded)."""
        if not args.sharded:
            h.set_gb300_options(L.gb300_options(chi0_precision=prec, device=local, reuse_device_inputs=reuse))
            e, _ = h.get_rpa_correlation_energy(opts, nq)
            return e, h.stats()
        from librpa_gb300.tau_shard import sharded_correlation_energy
        sts = []
        e, _ = sharded_correlation_energy(h, opts, nq, stats=sts, chi0_precision=prec, device=local,
                                          reuse_device_inputs=reuse)
        st = dict(sts[0])
        for k, v in sts[1].items():
            if k.startswith("t_") or k in ("n_launches", "dt_chi0_kernel_ms", "n_chi0_kernel", "chi0_flops",
                                           "ec_flops", "h2d_bytes", "d2h_bytes"):
                st[k] = st[k] + v
        return e, st

    ec = None
    for _ in range(max(args.warmup, 1)):
        ec, _ = step(1)
    # ---- device-resident timed region
    torch.cuda.synchronize()
    _barrier(dist)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches = 0
    chi0_ms, chi0_n, chi0_flops = 0.0, 0, 0.0
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            lib.librpa_gb300_clear_grid_cache()  # every step fits its minimax grids, as the reference does
            ec, st = step(1)
            launches += st["n_launches"]
            chi0_ms += st["dt_chi0_kernel_ms"]
            chi0_n += st["n_chi0_kernel"]
            chi0_flops += st["chi0_flops"]
        e1.record()
        torch.cuda.synchronize()
    _barrier(dist)
    ms = e0.elapsed_time(e1) / args.steps
    ms = _max_over_ranks(dist, ms)
    # ---- e2e: host buffers, re-staged every step
    step(0)
    torch.cuda.synchronize()
    _barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        lib.librpa_gb300_clear_grid_cache()
        ec2, st2 = step(0)
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    e2e_ms = _max_over_ranks(dist, e2e_ms)
    # ---- FP64 plain GPU path (the metric's denominator) and accuracy
    fp64 = None
    if args.fp64_check != "off" and prec != 0:
        est = chi0_flops / args.steps / 1.0e12  # seconds at ~1 TFLOP/s FP64
        if args.fp64_check == "on" or est < args.fp64_budget_s:
            # the plain FP64 GPU path: FP64 chi0 kernels and the all-FP64 Cholesky-form E_c (FP64
            # GEMMs for L^H chi0 L, batched FP64 Cholesky)
            h.set_gb300_options(L.gb300_options(chi0_precision=0, ec_path=L.EC_CHOL_FP64, device=local,
                                                reuse_device_inputs=1))
            t0 = time.perf_counter()
            e64, _ = h.get_rpa_correlation_energy(opts, nq)
            t64 = time.perf_counter() - t0
            fp64 = {"seconds": t64, "ec": e64, "dEc_meV_per_atom": abs(ec - e64) / s.n_atoms / (MEV_PER_ATOM_HA * 10),
                    "speedup": t64 / (ms / 1e3)}
        else:
            fp64 = {"skipped": f"estimated {est:.0f} s > budget {args.fp64_budget_s} s"}
    if rank != 0:
        return
    peaks, src = _peaks()
    bound = "tensor" if prec == 1 else "simt"
    peak = peaks.get("bf16_tflops", 1900.0) if prec == 1 else None
    ach = (chi0_flops / args.steps) / (chi0_ms / args.steps / 1e3) / 1e12 if chi0_ms > 0 else None
    roof = {"bound": "tensor", "achieved": ach, "peak": peaks.get("bf16_tflops"), "unit": "TFLOP/s",
            "frac": (ach / peaks.get("bf16_tflops")) if ach else None,
            "traffic": PROFILED_TRAFFIC.get(s.name, {}).get("bytes"),
            "traffic_source": PROFILED_TRAFFIC.get(s.name, {}).get("source"),
            "kernel": "chi0 contraction (X GEMMs + T1/T2 block contraction), per (tau, spin)",
            "flops_per_launch": chi0_flops / max(chi0_n, 1), "ms_per_launch": chi0_ms / max(chi0_n, 1),
            "peak_source": f"{src} bf16_tflops (burst)", "path": args.precision}
    cpu = None
    if ws == 1 and not args.no_cpu_baseline:
        v, desc = cpu_sample(s)
        cpu = {"value": v, "unit": "s", "cores": os.cpu_count(), "kind": "port", "sample": desc}
    line = {
        "metric": "rpa_ec_wall_time", "value": ms / 1e3, "unit": "s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "strong" if args.sharded else "weak",
        "vs_baseline": None, "dtype": {"bf16x3": "bf16x3/f32acc+f64", "fp32": "f32+f64", "fp64": "f64"}[args.precision],
        "data": "synthetic",
        "precision": args.precision,
        "parallelism": f"tau/q shards x{ws} (one reduce-scatter of chi0(q, omega))" if args.sharded else f"replicas x{ws}",
        "config": _config(s),
        "ec": ec, "chi0_tflops": ach, "chi0_flops_per_step": chi0_flops / args.steps,
        "t1_choice": {"narrow_producers": st["t1_narrow"], "kparts": st["t1_kparts"]},
        "stage_s": {k: st2[k] for k in ("t_grids", "t_upload", "t_gf", "t_chi0", "t_ftct", "t_ec", "t_total")},
        "fp64_gpu": fp64,
        "e2e": {"value": e2e_ms / 1e3, "unit": "s", "h2d_bytes_per_step": st2["h2d_bytes"],
                "d2h_bytes_per_step": st2["d2h_bytes"]},
        "gpu_launches": launches,
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
    }
    del h
    if ws == 1 and args.sc256:
        line["sc256_g"] = run_sc256(L, lib, torch, local, args)
    print(json.dumps(line), flush=True)


def run_sc256(L, lib, torch, local, args):
    """The 256-atom Gamma cell (13 NAO / 40 ABF per atom, C decay 1.5 A, 16 minimax points): the
    default path over 3 timed steps (grids fitted every step), the plain FP64 GPU path once (the
    denominator of the wall-time target), and the block-screened paths: the plain threshold
    rule at 1e-6 and the learned screening (trained on the plain run's logged blocks, 2% audit)."""
    from librpa_gb300 import synthetic as sy
    s = sy.sc256_g()
    opts = _opts(L, s)
    h = L.Handler()
    L.load_system(h, s)
    h.set_gb300_options(L.gb300_options(chi0_precision=1, device=local, reuse_device_inputs=1))
    h.get_rpa_correlation_energy(opts, 1)
    torch.cuda.synchronize()
    steps = 3
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        lib.librpa_gb300_clear_grid_cache()
        ec, _ = h.get_rpa_correlation_energy(opts, 1)
    e1.record()
    torch.cuda.synchronize()
    t_fast = e0.elapsed_time(e1) / steps / 1e3
    st = h.stats()
    out = {"workload": s.name, "n_atoms": s.n_atoms, "n_abf": int(sum(s.nabf)), "steps": steps,
           "seconds": t_fast, "ec": ec, "stage_s": {k: st[k] for k in ("t_gf", "t_chi0", "t_ftct", "t_ec")},
           "chi0_tflops": st["chi0_flops"] / (st["dt_chi0_kernel_ms"] / 1e3) / 1e12 if st["dt_chi0_kernel_ms"] else None}
    if args.fp64_check != "off":
        h.set_gb300_options(L.gb300_options(chi0_precision=0, ec_path=L.EC_CHOL_FP64, device=local,
                                            reuse_device_inputs=1))
        lib.librpa_gb300_clear_grid_cache()
        t0 = time.perf_counter()
        e64, _ = h.get_rpa_correlation_energy(opts, 1)
        t64 = time.perf_counter() - t0
        out["fp64_gpu"] = {"seconds": t64, "ec": e64, "speedup": t64 / t_fast,
                           "dEc_meV_per_atom": abs(ec - e64) / s.n_atoms / (MEV_PER_ATOM_HA * 10)}
    # block screening: plain threshold rule (logs the training blocks), then the learned predictor
    thr = 1e-6
    h.set_gb300_options(L.gb300_options(chi0_precision=1, device=local, reuse_device_inputs=1,
                                        screen_mode=L.SCREEN_THRESHOLD, screen_threshold=thr))
    t0 = time.perf_counter()
    e_plain, _ = h.get_rpa_correlation_energy(opts, 1)
    t_plain = time.perf_counter() - t0
    import ctypes
    rmse = ctypes.c_double()
    t0 = time.perf_counter()
    rc = lib.librpa_gb300_train_screening(h.h, 800, 3e-3, ctypes.byref(rmse))
    t_train = time.perf_counter() - t0
    if rc == 0:
        h.set_gb300_options(L.gb300_options(chi0_precision=1, device=local, reuse_device_inputs=1,
                                            screen_mode=L.SCREEN_MLP, screen_threshold=thr, audit_fraction=0.02,
                                            seed=7))
        lib.librpa_gb300_clear_grid_cache()
        t0 = time.perf_counter()
        e_mlp, _ = h.get_rpa_correlation_energy(opts, 1)
        t_mlp = time.perf_counter() - t0
        sm = h.stats()
        out["screening"] = {
            "threshold": thr, "plain_threshold_s": t_plain, "mlp_s": t_mlp, "train_s": t_train,
            "train_rmse_log10": rmse.value, "blocks_total": sm["blocks_total"],
            "blocks_computed": sm["blocks_computed"], "blocks_audited": sm["blocks_audited"],
            "fallbacks": sm["screen_fallbacks"],
            "dEc_vs_plain_meV_per_atom": abs(e_mlp - e_plain) / s.n_atoms / (MEV_PER_ATOM_HA * 10),
            "dEc_vs_unscreened_meV_per_atom": abs(e_mlp - ec) / s.n_atoms / (MEV_PER_ATOM_HA * 10)}
    del h
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="fcc16_k333")
    ap.add_argument("--precision", default="bf16x3", choices=list(PREC))
    ap.add_argument("--fp64-check", default="auto", choices=["auto", "on", "off"])
    ap.add_argument("--fp64-budget-s", type=float, default=90.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sharded", action="store_true",
                    help="split one E_c over the ranks (tau slices, a q-keyed reduce-scatter, q slices) "
                         "instead of running independent replicas")
    ap.add_argument("--no-sc256", dest="sc256", action="store_false",
                    help="skip the 256-atom sub-record (default path, FP64 denominator, screening)")
    args = ap.parse_args()
    ws, rank, local, dist = _dist()
    from librpa_gb300 import synthetic as sy
    s = sy.WORKLOADS[args.workload]()
    if args.impl == "reference":
        run_reference(args, s, ws, rank, dist)
    else:
        run_gb300(args, s, ws, rank, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
