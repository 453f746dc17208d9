"""Benchmark of the split-step evolution (libcugpe's gpe_evolve_qf path) on GB300.

Workload (one condensate per GPU): 128^3 unitary Fermi gas (dimers), real-time
evolution with quantum friction 0.1, dx = 0.2, trap omega = (1, 1, 1.5),
dt = 5e-3 (lattice dt' = 0.125), npart = 1000, starting from an imaginary-time
relaxed Thomas-Fermi state with the vortex phase atan2(y, x) imprinted.
Synthetic, seeded (numpy PCG64, seed 0).

A timed step is one gpe_evolve_qf(BLOCK) call (BLOCK GPE time steps, default
100) of the FP32-mixed engine; L2 is flushed (256 MiB write) before every timed
step.  `value` is GPE time steps per second with the state resident in HBM;
`e2e` is the same through the C ABI with host buffers: gpe_set_psi (host
complex128 -> device), gpe_evolve_qf(BLOCK), gpe_get_psi (device -> host).
The plain FP64 drop-in, the FP32 energy error against it, the reference
libcugpe engine on the same GPU (when its edited sources are present) and the
CPU FP64 oracle are reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

B_ALG = {  # algorithmic bytes per grid point per step (8 S + S + 4 s_r, + 4 S with quantum friction)
    ("fp32", True): 120, ("fp32", False): 88, ("fp64", True): 240, ("fp64", False): 176,
}
# warp instructions of one GPE step of the 128^3 FP32 friction step in the yz-plane layout (ncu
# smsp__inst_executed.sum over its four launches, profiles/plane_and_pass_kernel_issue_bound_128_fp32_ufg_qf.md)
INST_PER_STEP_128_PLANE = 58.4e6


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def fp64_rooflines(steps_per_s, n_points, fp64_peak, qf=True):
    """Both bounds of the FP64 form at `steps_per_s`: HBM (B_alg bytes per point per step) and the FP64
    ALU (F_alg = n_fft 5 N log2 N + 60 N flops per step: n_fft = 6 3D-transform equivalents with quantum
    friction -- the 18 axis transforms the engine runs, the friction Laplacian computed once per step --
    and 4 without, plus the pointwise phases).  `fp64_peak` = (TFLOP/s, kind).  The binding bound is the
    larger fraction."""
    hbm, kind = peaks()
    gbs = B_ALG[("fp64", qf)] * n_points * steps_per_s / 1e9
    n_fft = 6 if qf else 4
    flops = n_fft * 5.0 * n_points * float(np.log2(n_points)) + 60.0 * n_points
    tf = flops * steps_per_s / 1e12
    peak_tf, peak_kind = fp64_peak
    return {"hbm": {"achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm, "peak_kind": kind},
            "fp64_alu": {"achieved": tf, "peak": peak_tf, "unit": "TFLOP/s", "frac": tf / peak_tf,
                         "peak_kind": peak_kind, "flops_per_step": flops, "fft_equivalents_per_step": n_fft}}


def measured_fp64_peak():
    """FP64 FMA rate of this GPU measured now (independent DFMA chains, CUDA events)."""
    import libcugpe_gb300 as g
    try:
        return g.fp64_fma_rate(), "measured (DFMA-chain kernel, best of 5 launches, this run)"
    except Exception as ex:  # reported, never fatal
        return 1.25, f"nominal (measurement failed: {str(ex)[:80]})"


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="gpe_clocks_", suffix=".csv")
        os.close(fd)

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        # wait (3 s at most) for the first sample, so that sampling covers all the work that follows
        deadline = time.time() + 3.0
        while self.proc is not None and self.proc.poll() is None and time.time() < deadline:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=10)
        if getattr(self, "fh", None):
            self.fh.close()
        with open(self.path) as fh:
            self.lines = fh.read().splitlines()
        os.unlink(self.path)

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in getattr(self, "lines", []):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax = float(f[1])
            except ValueError:
                continue
            for name, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    """Replicas only: one independent condensate per rank, no data-path collective."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(ws, units_per_rank, seconds_this_rank):
    """Units all ranks processed / the slowest rank's time (weak scaling over replicas)."""
    return ws * units_per_rank / max_over_ranks(ws, seconds_this_rank)


def traffic_from_profiles(n):
    """DRAM bytes per GPE step of the pass kernels for this lattice, from the ncu summary under
    profiles/ ((bytes, how it was captured) or (None, None))."""
    path = os.path.join(ROOT, "profiles", "pass_kernel_traffic.txt")
    try:
        for line in open(path):
            f = line.split(None, 2)
            if len(f) >= 2 and f[0] == f"fp32_ufg_qf_rte_{n}":
                return float(f[1]), (f[2].strip() if len(f) > 2 else "")
    except OSError:
        pass
    return None, None


def workload(n):
    from libcugpe_gb300 import configs
    return configs.ufg_vortex_rte_qf(n=n)


def relaxed_state(w, ite_steps):
    """Imaginary-time relaxation of the Thomas-Fermi start, then the vortex phase."""
    import libcugpe_gb300 as g
    from libcugpe_gb300 import configs
    amp = np.abs(w.psi0)
    e = g.Engine(w.shape, w.interactions, 0.0, 1.0, w.dt, w.npart, precision=g.FP32)
    e.set_user_params(w.params)
    e.set_psi(0.0, amp)
    e.evolve_qf(ite_steps)
    _, psi = e.get_psi()
    e.close()
    X, Y, _ = configs.grid(w.shape)
    return np.abs(psi) * np.exp(1j * np.arctan2(Y + 0.5, X + 0.5))


def make_engine(w, psi, precision):
    import libcugpe_gb300 as g
    e = g.Engine(w.shape, w.interactions, w.alpha, w.beta, w.dt, w.npart, precision=precision)
    e.set_user_params(w.params)
    e.set_quantum_friction_coeff(w.qf)
    e.set_psi(0.0, psi)
    return e


def time_blocks(e, block, steps, warmup, flush, torch):
    """Device time of `steps` evolve_qf(block) calls, L2 flushed before each."""
    stream = torch.cuda.ExternalStream(e.stream_handle())
    for _ in range(warmup):
        e.evolve_qf(block)
    torch.cuda.synchronize()
    total = 0.0
    l0 = e.kernel_launches()
    for _ in range(steps):
        flush.add_(1.0)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        e.evolve_qf(block)
        b.record(stream)
        b.synchronize()
        total += a.elapsed_time(b) / 1e3
    return total, e.kernel_launches() - l0


def time_e2e(e, block, steps, host_psi, flush, torch):
    """The same through the C ABI with host buffers (H2D + evolve + D2H per step)."""
    stream = torch.cuda.ExternalStream(e.stream_handle())
    total = 0.0
    for _ in range(steps):
        flush.add_(1.0)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        e.set_psi(0.0, host_psi)
        e.evolve_qf(block)
        e.get_psi(out=host_psi)
        b.record(stream)
        b.synchronize()
        total += a.elapsed_time(b) / 1e3
    return total


def cpu_baseline(w, psi, seconds=15.0):
    """The CPU FP64 oracle on all host threads, a bounded number of steps."""
    import oracle
    threads = len(os.sched_getaffinity(0))
    o = oracle.Oracle(w.shape, w.interactions, w.alpha, w.beta, w.dt, w.npart, threads=threads)
    o.set_user_params(w.params)
    o.set_quantum_friction_coeff(w.qf)
    o.set_psi(0.0, psi)
    o.evolve_qf(1)
    steps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds or steps < 2:
        o.evolve_qf(1)
        steps += 1
    dt = time.perf_counter() - t0
    return {"value": steps / dt, "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} steps of the {w.shape[0]}^3 workload in {dt:.1f} s (oracle/gpe_oracle.c, FP64, OpenMP)"}


def reference_gpu(w, psi, steps=20):
    """The reference libcugpe engine (cuFFT Z2Z, FP64) built for this GPU, if its sources are here."""
    try:
        from oracle import build_ref, ref_run
        if not ref_run.available():
            return None
        nx, ny, nz = w.shape
        build_ref.build_one(nx, ny, nz, w.interactions)
        out = ref_run.run(w.shape, w.interactions, w.alpha, w.beta, w.dt, w.npart, w.params, psi,
                          ["S5", f"B{steps}", f"B{steps}"], qf=w.qf)
        ms = min(out["time_ms"])
        return {"value": steps / (ms / 1e3), "unit": "steps/s", "dtype": "f64",
                "what": "reference libcugpe dev/ engine (cuFFT Z2Z) built for sm_103a, CUDA events around gpe_evolve_qf"}
    except Exception as ex:  # reported, never fatal
        return {"unavailable": str(ex)[:200]}


def run_reference_arm(args, ws, rank):
    """--impl reference: the reference path timed on the host cores (the oracle port)."""
    if rank != 0:
        return
    w = workload(args.n)
    import oracle
    threads = len(os.sched_getaffinity(0))
    o = oracle.Oracle(w.shape, w.interactions, w.alpha, w.beta, w.dt, w.npart, threads=threads)
    o.set_user_params(w.params)
    o.set_quantum_friction_coeff(w.qf)
    o.set_psi(0.0, w.psi0)
    per = max(1, args.cpu_steps)
    for _ in range(args.warmup):
        o.evolve_qf(1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.evolve_qf(per)
    dt = time.perf_counter() - t0
    v = args.steps * per / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": config_obj(w, args),
            "cpu_baseline": {"value": v, "unit": "steps/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} x {per} steps of the {w.shape[0]}^3 workload "
                                       "(oracle/gpe_oracle.c FP64 restatement; the reference has no CPU path)"},
            "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


METRIC = "128^3 GPE steps/s (FP32-mixed split-step, UFG + quantum friction RTE)"


def config_obj(w, args):
    return {"workload": f"{w.shape[0]}^3 unitary Fermi gas RTE + quantum friction 0.1, dx=0.2, dt=5e-3, "
                        f"omega=(1,1,1.5), npart=1000, vortex start",
            "lattice": list(w.shape), "gpe_steps_per_timed_step": args.block, "precision": "fp32-mixed",
            "l2": "flushed (256 MiB write) before every timed step; the 128^3 FP32 working set stays in L2 within a step",
            "parallelism": f"replicas x{args.gpus}"}


def batch_ensemble(seed=0, counts=((32, 32), (64, 48), (128, 16)), box=16.0, dt=5e-3):
    """Ensemble of independent BEC ground-state problems of uneven lattice size.

    Per condensate: g N ~ U[50, 500], omega_z / omega_perp ~ U[0.8, 1.25],
    initial Gaussian width ~ U[0.8, 1.2] (oscillator units, omega_perp = 1), on
    a box of side `box` (dx = box / n), ITE time step dt (lattice dt / dx^2).
    """
    from libcugpe_gb300 import configs
    rng = np.random.default_rng(seed)
    out = []
    for n, c in counts:
        for _ in range(c):
            gN, ratio, width = rng.uniform(50, 500), rng.uniform(0.8, 1.25), rng.uniform(0.8, 1.2)
            dx = box / n
            shape = (n, n, n)
            X, Y, Z = configs.grid(shape, dx)
            psi = np.exp(-(X * X + Y * Y + Z * Z) / (2 * width * width)) * (1 + 0.01 * rng.uniform(-1, 1, shape))
            psi = configs.normalise(psi.astype(np.complex128), 1.0, 1.0)
            w = dx * dx
            params = [w, w, ratio * w, gN / dx / (4 * np.pi)]
            out.append({"shape": shape, "dx": dx, "dt": dt / (dx * dx), "params": params, "psi": psi})
    return out


def solve_until(evolve, chem, dx2, tol, check, max_steps):
    """Steps in chunks of `check` until the interval-mean mu changes by less than
    tol per step (physical units) between consecutive chunks, or max_steps."""
    steps, prev_sum, prev_mean = 0, None, None
    while steps < max_steps:
        evolve(check)
        steps += check
        mu, mu_sum = chem()
        if prev_sum is not None:
            mean = (mu_sum - prev_sum) / check
            if prev_mean is not None and abs(mean - prev_mean) / check / dx2 < tol:
                return steps, mean / dx2
            prev_mean = mean
        prev_sum = mu_sum
    return steps, None


def run_batch_workload(args):
    """Batched FP32-mixed ITE ensemble against a serial FP64 loop (JSON line)."""
    import torch
    import libcugpe_gb300 as g
    torch.cuda.set_device(0)
    ens = batch_ensemble()
    tol, check, max_steps = 1e-8, 25, args.batch_max_steps
    b = g.Batch([c["shape"] for c in ens], interactions=-1, alpha=0.0, beta=1.0, dt=[c["dt"] for c in ens])
    for i, c in enumerate(ens):
        b.engines[i].set_user_params(c["params"])
        b.engines[i].set_psi(0.0, c["psi"])
    dx2 = np.array([c["dx"] ** 2 for c in ens])
    # launch configuration of the batched passes chosen by the autotuner (state restored afterwards)
    t_tune = time.perf_counter()
    tuned = b.autotune(16)
    t_tune = time.perf_counter() - t_tune
    torch.cuda.synchronize()
    l0 = b.kernel_launches()
    t0 = time.perf_counter()
    # convergence test on the device: the interval mean of mu (lattice units) changes by < tol dx^2 per
    # step between consecutive intervals of `check` steps; a converged condensate is retired at once
    steps, mu_lat = b.solve(max_steps, check, tol * dx2)
    t_batch = time.perf_counter() - t0
    launches = b.kernel_launches() - l0
    done = steps >= 0
    mu_final = np.where(done, mu_lat / dx2, np.nan)
    # the unconverged, and what FP64 needs on the same problem
    stragglers = []
    for i in np.nonzero(~done)[0][: args.batch_diag]:
        c = ens[i]
        e = g.Engine(c["shape"], -1, 0.0, 1.0, c["dt"], 1.0, precision=g.FP64)
        e.set_user_params(c["params"])
        e.set_psi(0.0, c["psi"])
        st64, mu64 = solve_until(e.evolve_qf, e.chemical_potential, c["dx"] ** 2, tol, check, max_steps)
        e.close()
        stragglers.append({"n": c["shape"][0], "gN": c["params"][3] * c["dx"] * 4 * np.pi,
                           "omega_ratio": c["params"][2] / c["params"][0], "fp32_steps": int(max_steps),
                           "fp64_steps_to_converge": int(st64),
                           "fp32_vs_fp64_mu": float(abs(mu_lat[i] / dx2[i] - mu64) / abs(mu64)) if mu64 else None})
    # serial FP64 loop: one condensate at a time, same criterion; a stated subset per size
    per_size = {}
    subset = args.batch_serial_subset
    for n in sorted({c["shape"][0] for c in ens}):
        idx = [i for i, c in enumerate(ens) if c["shape"][0] == n][:subset]
        times, errs = [], []
        for i in idx:
            c = ens[i]
            e = g.Engine(c["shape"], -1, 0.0, 1.0, c["dt"], 1.0, precision=g.FP64)
            e.set_user_params(c["params"])
            e.set_psi(0.0, c["psi"])
            t1 = time.perf_counter()
            _, mu64 = solve_until(e.evolve_qf, e.chemical_potential, c["dx"] ** 2, tol, check, max_steps)
            times.append(time.perf_counter() - t1)
            if mu64 is not None and np.isfinite(mu_final[i]):
                errs.append(abs(mu_final[i] - mu64) / abs(mu64))
            e.close()
        per_size[n] = {"count": sum(1 for c in ens if c["shape"][0] == n), "timed": len(idx),
                       "mean_s": float(np.mean(times)), "mu_rel_err_fp32_vs_fp64": float(max(errs)) if errs else None}
    t_serial = sum(v["count"] * v["mean_s"] for v in per_size.values())
    line = {"metric": "batched ITE ensemble solves/s (96 BEC ground states: 32x32^3, 48x64^3, 16x128^3); "
                      f"serial FP64 loop timed on the first {subset} condensates of each size, extrapolated",
            "value": len(ens) / t_batch, "unit": "solves/s", "n_gpus": 1, "higher_is_better": True,
            "dtype": "f32", "data": "synthetic (seeded)", "converged": int(done.sum()), "of": len(ens),
            "batch_seconds": t_batch, "steps_max": int(steps.max()), "gpu_launches": int(launches),
            "serial_fp64": {"value": len(ens) / t_serial, "unit": "solves/s", "seconds_extrapolated": t_serial,
                            "per_size": per_size,
                            "how": f"FP64 engine, one condensate at a time, first {subset} of each size timed; "
                                   "the others take the mean of their size"},
            "speedup_vs_serial_fp64": t_serial / t_batch,
            "autotune": dict(tuned, seconds=t_tune, note="not in batch_seconds"),
            "fp32_steps_to_converge": {str(n): [int(x) for x in np.percentile(steps[[j for j, c in enumerate(ens)
                                                  if c["shape"][0] == n and done[j]]], [50, 90, 100])]
                                       if any(done[j] for j, c in enumerate(ens) if c["shape"][0] == n) else None
                                       for n in sorted({c["shape"][0] for c in ens})},
            "unconverged": stragglers,
            "config": {"workload": "ensemble of 96 BEC ITE solves (32 at 32^3, 48 at 64^3, 16 at 128^3), gN~U[50,500], omega_z/omega_perp~U[0.8,1.25], "
                                   "width~U[0.8,1.2], box 16 (dx=16/n), dt=5e-3; converged when the mean of mu over a "
                                   "25-step interval changes by < 1e-8 per step between intervals"}}
    return line


def run_bec64_workload(args):
    """64^3 BEC imaginary-time ground state (FP64, 2000 steps, mu every step), against the
    reference engine on the same GPU and the CPU oracle."""
    import libcugpe_gb300 as g
    from libcugpe_gb300 import configs
    w = configs.bec_ground_state_ite(n=64, steps=2000)
    e = g.Engine(w.shape, -1, 0.0, 1.0, w.dt, w.npart, precision=g.FP64)
    e.set_user_params(w.params)
    e.set_psi(0.0, w.psi0)
    e.normalize_psi()
    e.evolve_qf(20)
    e.set_psi(0.0, w.psi0)
    e.normalize_psi()
    t0 = time.perf_counter()
    mu = e.evolve_qf(w.steps)
    t_ours = time.perf_counter() - t0
    en = e.energy()
    line = {"metric": "64^3 BEC ITE steps/s (FP64 drop-in)", "value": w.steps / t_ours, "unit": "steps/s",
            "n_gpus": 1, "higher_is_better": True, "dtype": "f64", "data": "synthetic (seeded)",
            "mu": mu, "energy_per_particle": sum(en[1:]),
            "config": {"workload": "contact-BEC ITE ground state: 64^3, dx=0.25, omega=1, gN=100, ITE dt=1e-3, 2000 steps, "
                                   "Gaussian width 1 x (1+0.01u)"}}
    try:
        from oracle import build_ref, ref_run
        if ref_run.available():
            build_ref.build_one(64, 64, 64, -1)
            out = ref_run.run(w.shape, -1, 0.0, 1.0, w.dt, w.npart, w.params, w.psi0,
                              ["N", "S20", "N", f"B{w.steps}", "E"])
            line["reference_gpu"] = {"value": w.steps / (out["time_ms"][0] / 1e3), "unit": "steps/s",
                                     "what": "reference libcugpe (cuFFT Z2Z) for sm_103a, mu requested every step "
                                             "(its synchronous D2H per step)"}
    except Exception as ex:
        line["reference_gpu"] = {"unavailable": str(ex)[:200]}
    return line


def run_cool512_workload(args):
    """Large cooling run (512^3, dx=0.1, UFG + quantum friction 0.2, FP32, 8 vortex lines, dt=2e-3,
    5000 steps): steps/s, HBM roofline, and the final energy against an FP64 run of the 256^3
    lattice subsampled from the same initial state (dx=0.2, same physical time)."""
    import torch
    import libcugpe_gb300 as g
    from libcugpe_gb300 import configs
    w = configs.ufg_vortex_lines(n=args.n if args.n != 128 else 512, steps=args.cool_steps)
    dx = 0.1 * 512 / w.shape[0]
    e = g.Engine(w.shape, 0, 1.0, 0.0, w.dt, w.npart, precision=g.FP32)
    e.set_user_params(w.params)
    e.set_quantum_friction_coeff(w.qf)
    e.set_psi(0.0, w.psi0)
    e0 = sum(e.energy()[1:]) / dx ** 2
    # launch configuration chosen by the autotuner (radix plan per fused pass, graph length), outside
    # the timed region; it restores psi, time and step counter
    t_tune = time.perf_counter()
    tuned = e.autotune(8)
    t_tune = time.perf_counter() - t_tune
    stream = torch.cuda.ExternalStream(e.stream_handle())
    with Clocks(0) as clk:
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        e.evolve_qf(w.steps)
        b.record(stream)
        b.synchronize()
    secs = a.elapsed_time(b) / 1e3
    e1 = sum(e.energy()[1:]) / dx ** 2
    passes = e.profile_passes(5)
    e.close()
    # FP64 on the 256^3 lattice subsampled from the same initial state (every other point)
    n2 = w.shape[0] // 2
    psi2 = configs.normalise(np.ascontiguousarray(w.psi0[::2, ::2, ::2]), w.npart, 2.0)
    dx2 = 2 * dx
    f = g.Engine((n2, n2, n2), 0, 1.0, 0.0, w.dt / 4.0, w.npart, precision=g.FP64)
    f.set_user_params([p * 4.0 for p in w.params[:3]] + [0.0])
    f.set_quantum_friction_coeff(w.qf)
    f.set_psi(0.0, psi2)
    f0 = sum(f.energy()[1:]) / dx2 ** 2
    t0 = time.perf_counter()
    f.evolve_qf(w.steps)
    t64 = time.perf_counter() - t0
    f1 = sum(f.energy()[1:]) / dx2 ** 2
    f.close()
    n = int(np.prod(w.shape))
    peak, kind = peaks()
    achieved = B_ALG[("fp32", True)] * n * w.steps / secs / 1e9
    line = {"metric": "512^3 GPE steps/s (FP32-mixed, UFG + quantum friction 0.2, 8 vortex lines)",
            "value": w.steps / secs, "unit": "steps/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded)", "points_steps_per_s": n * w.steps / secs,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "basis": "B_alg 120 B/pt/step, whole evolve_qf(%d) timed with CUDA events; peak %s"
                                  % (w.steps, kind),
                         "per_pass_us": [round(p["ms"] * 1e3, 1) for p in passes]},
            "energy_per_particle_osc_units": {"fp32_512_initial": e0 / w.npart, "fp32_512_final": e1 / w.npart,
                                              "fp64_256_initial": f0 / w.npart, "fp64_256_final": f1 / w.npart,
                                              "final_rel_diff": abs(e1 - f1) / abs(f1)},
            "fp64_256_seconds": t64, "clocks": clk.summary(),
            "autotune": dict(tuned, seconds=t_tune, note="before the timed run, state restored"),
            "config": {"workload": "cooling run: 512^3, dx=0.1, UFG, quantum friction 0.2, omega=1, 8 vortex lines "
                                   "(charge +1, seeded in the disk r<4), dt=2e-3, %d steps, npart=5e4"
                                   % w.steps, "lattice": list(w.shape)}}
    return line


def run_control_workload(args):
    """Optimal control, 64^3 real-time BEC (gN=200, dt=1e-3, 2000 steps, 16 Gaussians x 100 slices):
    adjoint gradient timing and its check against central differences at 20 seeded controls."""
    import libcugpe_gb300 as g
    from libcugpe_gb300 import configs
    from libcugpe_gb300.control import ControlProblem
    n, dx, gN, dt_phys, nsteps, nsl, nb, sigma = 64, 0.25, 200.0, 1e-3, args.control_steps, 100, 16, 0.8
    rng = np.random.default_rng(0)
    shape = (n, n, n)
    w = dx * dx
    params = [w, w, w, gN / dx / (4 * np.pi)]
    dt = dt_phys / (dx * dx)
    X, Y, Z = configs.grid(shape, dx)
    centres = rng.uniform(-3, 3, (nb, 3))
    basis = np.stack([np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) / (2 * sigma * sigma))
                      for c in centres]) * (dx * dx)  # lattice energy units per unit physical control
    c_phys = 0.05 * rng.standard_normal((nsl, nb))

    def ground_state(shift):
        e = g.Engine(shape, -1, 0.0, 1.0, dt * 20, 1.0, precision=g.FP64)
        e.set_user_params(params)
        if shift:  # trap centred at x = shift: 0.5 (x - s)^2 - 0.5 x^2 = -s x + s^2/2
            e.set_potential_slices(((-shift * X + 0.5 * shift * shift) * dx * dx)[None], 1)
        e.set_psi(0.0, configs.normalise(np.exp(-((X - shift) ** 2 + Y * Y + Z * Z) / 2).astype(np.complex128), 1, 1))
        for _ in range(40):
            e.evolve_qf(100)
        psi = e.get_psi()[1]
        e.close()
        return psi

    psi0, target = ground_state(0.0), ground_state(0.5)
    e = g.Engine(shape, -1, 1.0, 0.0, dt, 1.0, precision=g.FP64)
    e.set_user_params(params)
    cp = ControlProblem(e, basis, nsl, nsteps // nsl, nsteps, target, checkpoint_every=args.control_ckpt)
    t0 = time.perf_counter()
    loss = cp.loss(c_phys, psi0)
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    loss2, grad = cp.loss_and_grad(c_phys, psi0)
    t_grad = time.perf_counter() - t0
    h = 1e-4
    errs = []
    picks = [(int(rng.integers(nsl)), int(rng.integers(nb))) for _ in range(args.control_fd)]
    for s_, k_ in picks:
        cpl, cmi = c_phys.copy(), c_phys.copy()
        cpl[s_, k_] += h
        cmi[s_, k_] -= h
        fd = (cp.loss(cpl, psi0) - cp.loss(cmi, psi0)) / (2 * h)
        errs.append({"slice": s_, "basis": k_, "adjoint": float(grad[s_, k_]), "fd": float(fd),
                     "rel_err": float(abs(fd - grad[s_, k_]) / max(abs(grad[s_, k_]), 1e-30))})
    line = {"metric": "optimal-control loss+gradient (64^3 RTE BEC, 2000 steps, 1600 controls) per second",
            "value": 1.0 / t_grad, "unit": "gradients/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f64",
            "data": "synthetic (seeded)", "loss": loss2, "loss_forward_only": loss, "forward_seconds": t_fwd,
            "forward_plus_adjoint_seconds": t_grad, "grad_norm": float(np.linalg.norm(grad)),
            "fd_check": {"h": h, "controls": len(errs), "max_rel_err": max(e_["rel_err"] for e_ in errs),
                         "median_rel_err": float(np.median([e_["rel_err"] for e_ in errs])), "points": errs},
            "config": {"workload": "optimal control of an RTE BEC: 64^3, dx=0.25, gN=200, omega=1, dt=1e-3, 2000 steps, 16 Gaussians "
                                   "sigma=0.8 centres U[-3,3]^3, 100 slices, controls N(0,0.05), target = ground state "
                                   "of the trap shifted by (0.5,0,0), checkpoints every 100 steps"}}
    cp.close()
    return line


def run_lattice_workload(args):
    """A seeded FP32-mixed (or FP64) UFG + quantum friction real-time run on any lattice, for kernel
    profilers: `--warm` steps (the first step runs 8 fused passes, every later one 7), then `--steps`
    more, so that `ncu -k regex:pass_kernel -s <7*warm+1> -c <7*steps>` captures whole steady steps."""
    import libcugpe_gb300 as g
    from libcugpe_gb300 import configs
    shape = tuple(int(x) for x in args.lattice.split(","))
    prec = g.FP32 if args.precision == "fp32" else g.FP64
    e = g.Engine(shape, 0, 1.0, 0.0, 0.02, 1e5, precision=prec)
    if args.plan:
        e.set_fft_plan(args.plan)
    e.set_user_params([0.002, 0.002, 0.003, 0.0])
    e.set_quantum_friction_coeff(0.1)
    e.set_psi(0.0, configs.random_state(shape, seed=3, npart=1e5, gamma=2.0))
    e.evolve_qf(args.warm)
    e.synchronize()
    t0 = time.perf_counter()
    e.evolve_qf(args.steps)
    e.synchronize()
    secs = time.perf_counter() - t0
    e.close()
    return {"metric": "seeded run for profilers (wall clock, not a benchmark)", "lattice": list(shape),
            "precision": args.precision, "plan": args.plan, "steps": args.steps, "seconds": secs}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--block", type=int, default=100)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-extras", action="store_true", help="only the headline line (profiling runs)")
    ap.add_argument("--ite-steps", type=int, default=200)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--fp32-check-steps", type=int, default=10000)
    ap.add_argument("--workload", default="ufg_qf",
                    choices=["ufg_qf", "batch", "control", "bec64", "cool512", "lattice"])
    ap.add_argument("--lattice", default="512,512,128")
    ap.add_argument("--warm", type=int, default=3)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--plan", type=int, default=0, help="radix plan of the lattice workload's pencils (0 or 1)")
    ap.add_argument("--cool-steps", type=int, default=5000)
    ap.add_argument("--control-steps", type=int, default=2000)
    ap.add_argument("--control-ckpt", type=int, default=100)
    ap.add_argument("--control-fd", type=int, default=20)
    ap.add_argument("--batch-max-steps", type=int, default=20000)
    ap.add_argument("--batch-serial-subset", type=int, default=2)
    ap.add_argument("--batch-diag", type=int, default=4)
    args = ap.parse_args()
    single = {"batch": run_batch_workload, "control": run_control_workload, "bec64": run_bec64_workload,
              "cool512": run_cool512_workload, "lattice": run_lattice_workload}
    if args.workload in single:
        print(json.dumps(single[args.workload](args)), flush=True)
        return
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference_arm(args, ws, rank)
        return

    import torch
    import libcugpe_gb300 as g
    torch.cuda.set_device(local)
    w = workload(args.n)
    psi = relaxed_state(w, args.ite_steps)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    e32 = make_engine(w, psi, g.FP32)
    # launch configuration chosen by the autotuner (operand staging, graph length, radix plan per fused
    # pass), before the timed region; it restores psi, time and step counter
    tuned = e32.autotune(16)
    barrier(ws)
    with Clocks(local) as clk:
        t32, launches = time_blocks(e32, args.block, args.steps, args.warmup, flush, torch)
    value = whole_job_rate(ws, args.steps * args.block, t32)
    t32 = max_over_ranks(ws, t32)
    # per-pass kernel times (CUDA events around each fused pass, engine stream): shares of the step
    passes = e32.profile_passes(20)

    host = torch.empty(w.shape + (2,), dtype=torch.float64, pin_memory=True).numpy().view(np.complex128)[..., 0]
    host[...] = psi
    te2e = time_e2e(e32, args.block, max(2, args.steps // 2), host, flush, torch)
    e2e_value = whole_job_rate(ws, max(2, args.steps // 2) * args.block, te2e)

    extras = {}
    if not args.no_extras and rank == 0:
        # plain FP64 drop-in on the same workload, with both of its rooflines (FP64 peak measured now)
        e64 = make_engine(w, psi, g.FP64)
        b64 = max(5, args.block // 10)
        t64, _ = time_blocks(e64, b64, 3, 1, flush, torch)
        extras["fp64_plain"] = {"value": 3 * b64 / t64, "unit": "steps/s", "dtype": "f64",
                                "roofline": fp64_rooflines(3 * b64 / t64, int(np.prod(w.shape)),
                                                           measured_fp64_peak(), qf=w.qf != 0.0)}
        # the binding unit, counted by ncu on this workload's seven FP64 passes (one steady step of the
        # 128^3 friction schedule): every DADD/DMUL/DFMA, where fp64_alu counts nominal FFT flops
        if tuple(w.shape) == (128, 128, 128) and w.qf != 0.0:
            extras["fp64_plain"]["roofline"]["fp64_pipe"] = {
                "active_frac": 0.83, "per_pass": [0.819, 0.844, 0.835, 0.830, 0.832, 0.835, 0.842],
                "how": "ncu sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active, one steady step "
                       "of the 128^3 FP64 friction schedule (pass_kernel_fp64_pipe_128_ufg_qf.md)"}
        e64.close()
        # FP32 energy and density error against the FP64 form over the workload's full run
        a = make_engine(w, psi, g.FP32)
        b = make_engine(w, psi, g.FP64)
        nchk = args.fp32_check_steps
        a.evolve_qf(nchk)
        b.evolve_qf(nchk)
        ea, eb = a.energy(), b.energy()
        Ea, Eb = sum(ea[1:]), sum(eb[1:])
        _, da = a.get_density()
        _, db = b.get_density()
        extras["fp32_vs_fp64"] = {"steps": nchk, "dE_over_E": abs(Ea - Eb) / abs(Eb),
                                  "density_rel_l2": float(np.linalg.norm(da - db) / np.linalg.norm(db))}
        a.close(); b.close()
        # the workload with its Weizsaecker gradient term of weight 0.25 (not in the reference:
        # pinned by the oracle only); FP32 speed and FP32-vs-FP64 error after the same steps
        aw = make_engine(w, psi, g.FP32)
        aw.set_weizsacker(0.25)
        tw, _ = time_blocks(aw, args.block, max(2, args.steps // 2), 1, flush, torch)
        aw.set_psi(0.0, psi)
        bw = make_engine(w, psi, g.FP64)
        bw.set_weizsacker(0.25)
        nwz = 200
        aw.evolve_qf(nwz)
        bw.evolve_qf(nwz)
        ea, eb = aw.energy(), bw.energy()
        Ea, Eb = sum(ea[1:]), sum(eb[1:])
        _, da = aw.get_density()
        _, db = bw.get_density()
        extras["weizsacker_0.25"] = {
            "value": max(2, args.steps // 2) * args.block / tw, "unit": "steps/s", "dtype": "f32",
            "fp32_vs_fp64": {"steps": nwz, "dE_over_E_without_EW": abs(Ea - Eb) / abs(Eb),
                             "density_rel_l2": float(np.linalg.norm(da - db) / np.linalg.norm(db))}}
        aw.close(); bw.close()
        ref = reference_gpu(w, psi)
        if ref:
            extras["reference_gpu"] = ref
        extras["cpu_baseline"] = cpu_baseline(w, psi, seconds=args.cpu_seconds)
        # the other workloads of the benchmark set, each with its own value and checks
        for key, fn in (("bec64_ite", run_bec64_workload), ("batch_ensemble", run_batch_workload),
                        ("control_adjoint", run_control_workload), ("cool512", run_cool512_workload)):
            t_w = time.perf_counter()
            try:
                extras[key] = fn(args)
            except Exception as ex:  # reported, never fatal
                extras[key] = {"unavailable": f"{type(ex).__name__}: {str(ex)[:300]}"}
            extras[key]["wall_s"] = round(time.perf_counter() - t_w, 1)

    if rank == 0:
        n = int(np.prod(w.shape))
        peak, kind = peaks()
        # the roofline follows from the timed number: one GPE step = ms_per_step / block
        gpe_step_s = t32 / (args.steps * args.block)
        achieved = B_ALG[("fp32", True)] * n / gpe_step_s / 1e9
        # per-pass CUDA-event times (measured with an event between passes, which breaks the overlap of
        # programmatic dependent launch) serve as shares of the timed step
        ev_total = sum(p["ms"] for p in passes)
        per_pass = []
        for p in passes:
            share = p["ms"] / ev_total
            us = share * gpe_step_s * 1e6
            per_pass.append({"axis": p["axis"], "kind": p["kind"], "share": round(share, 4),
                             "us_in_step": round(us, 2), "own_bytes_GBps": round(p["bytes"] / (us / 1e6) / 1e9, 1)})
        top = max(per_pass, key=lambda p: p["share"])
        traffic, traffic_how = traffic_from_profiles(w.shape[0])
        clk_s = clk.summary()
        # the unit that binds the L2-resident 128^3 step: instruction issue (one warp instruction per
        # scheduler per cycle, four schedulers per SM, at the SM clock sampled during the timed region)
        issue = None
        if tuple(w.shape) == (128, 128, 128) and w.qf != 0.0 and any(p["kind"] == "plane" for p in passes):
            sms = torch.cuda.get_device_properties(local).multi_processor_count
            mhz = clk_s.get("sm_mhz") or clk_s.get("sm_max_mhz") or 2070.0
            peak_inst = sms * 4 * mhz * 1e6
            ach_inst = INST_PER_STEP_128_PLANE / gpe_step_s
            issue = {"unit": "warp instructions/s", "achieved": ach_inst, "peak": peak_inst,
                     "frac": ach_inst / peak_inst, "inst_per_gpe_step": INST_PER_STEP_128_PLANE,
                     "how": f"ncu instruction count per GPE step / timed GPE step; peak = {sms} SMs x 4 "
                            f"schedulers x {mhz:.0f} MHz (plane_and_pass_kernel_issue_bound_128_fp32_ufg_qf.md)"}
        line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * t32 / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": config_obj(w, args),
                "points_steps_per_s": value * n,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic, "traffic_how": traffic_how,
                             "kernel": "plane_kernel + pass_kernel (two yz-plane passes and two x-pencil passes per GPE step)",
                             "basis": f"B_alg {B_ALG[('fp32', True)]} B/pt/step x {n} pts / {1e6 * gpe_step_s:.2f} us "
                                      f"per GPE step (= ms_per_step / {args.block}, CUDA events on the engine "
                                      f"stream); peak {kind}; traffic = ncu DRAM bytes per GPE step",
                             "per_pass": per_pass,
                             "top_pass": top,
                             "per_pass_event_sum_us": round(1e3 * ev_total, 2),
                             "issue": issue},
                "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": 16 * n,
                        "d2h_bytes_per_step": 16 * n},
                "gpu_launches": launches, "clocks": clk_s, "autotune": tuned}
        line.update(extras)
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
