#!/usr/bin/env python
"""Throughput of the hydrodynamic step (steps/s) on one GB300.

Workload: N = 2048 monodisperse spheres, volume fraction 0.5, seeded minimum
gap 1e-4 a, Lees-Edwards shear rate 1, dt = 5e-4, Ewald tolerance 1e-10,
lubrication on -- one STEPPER_Stokesian step per timed iteration, all
inputs resident in HBM.  The grand mobility alone (4.06 GB FP64) is larger
than L2, so no flush is needed between iterations.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision mixed|fp64] [--N 2048] [--phi 0.5]

Prints one JSON line (rank 0).  With --gpus N > 1 under torchrun every rank
steps its own independent replica (the step does not shard; replicas only).
--impl reference times the CPU restatement of the reference's routines on the
host cores instead (bounded samples, see cpu_step_sample()).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "steps/s N=2048 φ=0.5: mixed+learned vs plain FP64 on GB300, vel err ≤1e-8"
SEED_BASE = 20260000


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--N", type=int, default=2048)
    ap.add_argument("--phi", type=float, default=0.5)
    ap.add_argument("--gmin", type=float, default=1e-4)
    ap.add_argument("--dt", type=float, default=5e-4)
    ap.add_argument("--sweeps", type=int, default=200)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-peaks", action="store_true")
    ap.add_argument("--tensor-cores", type=int, default=1, choices=[0, 1, 3],
                    help="FP32 factorisations of the mixed form: 1 TF32/3xTF32 per factor, 3 all 3xTF32, 0 SIMT")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_seed(rank):
    """Seed of rank `rank`'s packing: every replica steps its own system."""
    return SEED_BASE + 5000 + rank


def max_over_ranks(x, ws, dist, torch, device):
    """Largest per-rank duration over all ranks.  Replicas exchange nothing
    on the data path; only the clock is reduced."""
    if ws <= 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(ws, steps, seconds):
    """Whole-job steps/s: every rank's steps over the slowest rank's time."""
    return ws * steps / seconds


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fp:
            return json.load(fp)
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region; the
    raw samples go to RSD_CLOCKS_DIR (default: the system's temporary
    directory), their summary into the JSON line."""

    def __init__(self, index):
        import tempfile
        self.index = index
        self.proc = None
        folder = os.environ.get("RSD_CLOCKS_DIR", tempfile.gettempdir())
        self.path = os.path.join(folder, "clocks_%d.csv" % os.getpid())

    def start(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.fp = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fp,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fp.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            v = [x.strip() for x in line.split(",")]
            if len(v) < 9:
                continue
            try:
                sm.append(float(v[1]))
                mx.append(float(v[2]))
            except ValueError:
                continue
            for nm, flag in zip(names, v[5:9]):
                if flag.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def fp64_gemm_peak(torch, dev):
    """cuBLAS DGEMM rate on this GPU (TFLOP/s): the denominator for the FP64
    kernels, since the measured-peaks file carries BF16 and HBM only."""
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    c = a @ b
    torch.cuda.synchronize(dev)
    best = 0.0
    for _ in range(2):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        c = a @ b
        e1.record()
        torch.cuda.synchronize(dev)
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b, c
    return best


def fp32_gemm_peak(torch, dev):
    """cuBLAS FP32 GEMM with TF32 tensor cores, TFLOP/s: the denominator for
    the FP32 factorisations of the mixed form, whose GEMMs run on tcgen05 in
    TF32 and 3xTF32 (the measured-peaks file carries BF16 and HBM only)."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    n = 8192
    a = torch.randn(n, n, dtype=torch.float32, device=dev)
    b = torch.randn(n, n, dtype=torch.float32, device=dev)
    c = a @ b
    torch.cuda.synchronize(dev)
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        c = a @ b
        e1.record()
        torch.cuda.synchronize(dev)
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    torch.backends.cuda.matmul.allow_tf32 = prev
    del a, b, c
    return best


def ewald_flops(N, NR, NI):
    """Algorithmic FLOP of one grand-mobility assembly: 500 per real image and
    150 per reciprocal vector, over the unordered pairs (all images) and the
    self terms (n != 0 and k != 0)."""
    nr = (2 * NR + 1) ** 3
    nk = (2 * NI + 1) ** 3 - 1
    pairs = N * (N - 1) // 2
    return pairs * (nr * 500.0 + nk * 150.0) + N * ((nr - 1) * 500.0 + nk * 150.0)


def solve_flops(N, precision):
    """Plain FP64: Cholesky + SPD inverse of M (n^3, n = 11N) and Cholesky of
    RPP ((6N)^3/3): 1403 N^3.  Mixed: FP32 Cholesky of M' (n^3/3), inverse of
    its 6N Schur factor (2 (6N)^3/3) and Cholesky of RPP ((6N)^3/3): 660 N^3."""
    if precision == "fp64":
        return 1403.0 * N ** 3
    return (1331.0 / 3.0 + 216.0) * N ** 3


def cpu_step_sample(pos, radii, L, N, dt, threads):
    """Seconds per step of the CPU restatement of the reference's routines at
    the full workload, from bounded samples:
      assembly  PER_GRPERY_INV_FRI on the first 96 particles in the full box
                (4560 pairs, same images per pair), scaled to N(N-1)/2 pairs
                plus N self terms;
      lub       lubmxcalc at N = 512 at the same volume fraction, scaled by
                (N/512)^2 (pair sweep and dense outputs are O(N^2));
      solve     LAPACK DPOTRF + DPOTRI of the 11*512 grand mobility plus DPOTRF
                of the 6*512 RPP block (scipy's OpenBLAS), scaled by (N/512)^3.
    Returns (seconds, description)."""
    from oracle import oracle as o
    from scipy.linalg import lapack

    mu = o.mu_f_dimensionless(1.0)
    lat = o.set_lattice_skew(0.0, [L, L, L], 1.0)
    ns = min(96, N)
    t0 = time.perf_counter()
    G, _ = o.per_grpery_inv_fri(pos[:ns], radii[:ns], lat, 1e-10, mu)
    t_asm = time.perf_counter() - t0
    pairs_s = ns * (ns - 1) / 2 + ns
    pairs = N * (N - 1) / 2 + N
    t_asm_full = t_asm * pairs / pairs_s
    n_l = min(512, N)
    lat2 = o.set_lattice_skew(0.0, [L, L, L], 1.0)
    tab = o.LubTab(os.path.join(ROOT, "tests", "golden", "lubdat"))
    # a 512-particle box at the same volume fraction
    L2 = L * (n_l / N) ** (1.0 / 3.0)
    sel = pos[np.all(pos < L2, axis=1)][:n_l] if N > n_l else pos
    lat2 = o.set_lattice_skew(0.0, [L2, L2, L2], 1.0)
    t0 = time.perf_counter()
    o.lubmxcalc(sel, np.ones(len(sel)), lat2, mu, tab)
    t_lub = (time.perf_counter() - t0) * (N / max(len(sel), 1)) ** 2
    n_s = 11 * n_l
    rng = np.random.default_rng(0)
    X = rng.standard_normal((n_s, n_s))
    A = np.asfortranarray(X @ X.T / n_s + np.eye(n_s))
    B = np.asfortranarray(A[:6 * n_l, :6 * n_l].copy())
    t0 = time.perf_counter()
    c, _ = lapack.dpotrf(A, lower=0, clean=0, overwrite_a=1)
    lapack.dpotri(c, lower=0, overwrite_c=1)
    lapack.dpotrf(B, lower=0, clean=0, overwrite_a=1)
    t_solve = (time.perf_counter() - t0) * (N / n_l) ** 3
    total = t_asm_full + t_lub + t_solve
    desc = ("port (C restatement + OpenBLAS LAPACK), %d threads; per step = assembly of %d particles' %d pairs "
            "scaled to %d, lub at N=%d scaled by N^2, DPOTRF+DPOTRI at n=%d scaled by n^3 "
            "(assembly %.1f s, lub %.2f s, solve %.1f s)" % (threads, ns, int(pairs_s), int(pairs), len(sel), n_s,
                                                           t_asm_full, t_lub, t_solve))
    return total, desc


def reference_arm(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    import __graft_entry__ as ge
    from oracle import oracle as o
    o.build()
    rsd_cfg = _configs()
    pos, radii, L = rsd_cfg.packing(args.N, args.phi, args.gmin, replica_seed(0), sweeps=args.sweeps)
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    for _ in range(args.warmup):
        cpu_step_sample(pos, radii, L, args.N, args.dt, threads)
    ts = []
    desc = ""
    for _ in range(args.steps):
        t, desc = cpu_step_sample(pos, radii, L, args.N, args.dt, threads)
        ts.append(t)
    sec = float(np.mean(ts))
    v = 1.0 / sec
    line = {"metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded sphere packing)",
            "config": {"workload": "STEPPER_Stokesian step, N=%d phi=%.2f gap>=%g, shear 1, dt %g, Ewald 1e-10, lub on"
                                   % (args.N, args.phi, args.gmin, args.dt), "l2": "inputs larger than L2"},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "steps/s", "cores": threads, "kind": "port", "sample": desc},
            "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _configs():
    import importlib.util
    path = os.path.join(ROOT, "regularized-stokesian-dynamics_gb300", "configs.py")
    spec = importlib.util.spec_from_file_location("rsd_configs_only", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
        return
    import torch
    import torch.distributed as dist

    import __graft_entry__ as ge

    ws, rank, local = dist_env()
    if ws > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    rsd = ge.load_package()
    prec = rsd.PREC_MIXED if args.precision == "mixed" else rsd.PREC_FP64
    pos, radii, L = rsd.configs.packing(args.N, args.phi, args.gmin, replica_seed(rank), sweeps=args.sweeps)
    N = args.N
    mu = rsd.mu_f_dimensionless(1.0)
    ctx = rsd.Context(local)
    ctx.set_tensor_cores(args.tensor_cores)
    tab = rsd.LubTab(rsd.lubdat_dir())
    conf_t = torch.tensor(pos, dtype=torch.float64, device=dev)
    radii_t = torch.tensor(radii, dtype=torch.float64, device=dev)
    U_t = torch.empty(6 * N, dtype=torch.float64, device=dev)
    S_t = torch.empty(5 * N, dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    T = 0.0
    stream = torch.cuda.ExternalStream(ctx.stream)
    lib = rsd.library()

    def step():
        nonlocal T
        y, info = rsd.stepper_stokesian_dev(ctx, tab, conf_t, radii_t, T, args.dt, [L, L, L], 1.0, mu, 1e-10, U_t, S_t,
                                            precision=prec)
        T += args.dt
        return y, info

    for _ in range(args.warmup):
        step()
    sampler = ClockSampler(local) if rank == 0 else None
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    if sampler:
        sampler.start()
    n0 = lib.rsd_launch_count() if hasattr(lib, "rsd_launch_count") else 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    phases = np.zeros(4)
    infos = []
    for _ in range(args.steps):
        y, info = step()
        phases += ctx.phase_ms()
        infos.append((info.NR, info.NI, info.iterations, info.residual))
    e1.record(stream)
    torch.cuda.synchronize(dev)
    launches = (lib.rsd_launch_count() - n0) if hasattr(lib, "rsd_launch_count") else None
    ms = e0.elapsed_time(e1)
    clocks = sampler.stop() if sampler else None
    ms = max_over_ranks(ms, ws, dist, torch, dev)
    ms_per_step = ms / args.steps
    value = replica_throughput(ws, args.steps, ms * 1e-3)
    # end to end through the host C-ABI call (H2D of the inputs, D2H of the results)
    e2e = None
    if not args.no_e2e:
        conf_h = conf_t.cpu().numpy().copy()
        t0 = time.perf_counter()
        Te = T
        for _ in range(args.steps):
            out = rsd.STEPPER_Stokesian(ctx, tab, conf_h, radii, Te, args.dt, [L, L, L], 1.0, mu, 1e-10,
                                        precision=prec)
            conf_h = out["conf"]
            Te += args.dt
        te = max_over_ranks(time.perf_counter() - t0, ws, dist, torch, dev)
        e2e = {"value": replica_throughput(ws, args.steps, te), "unit": "steps/s", "h2d_bytes_per_step": 8 * (3 * N + N),
               "d2h_bytes_per_step": 8 * (3 * N + 6 * N + 5 * N)}
    # the plain FP64 form on the same start configuration: its steps/s and the
    # mixed form's velocity / stresslet error against it
    plain = None
    if not args.no_plain and args.precision == "mixed":
        c0 = torch.tensor(pos, dtype=torch.float64, device=dev)
        Um, Sm = torch.empty_like(U_t), torch.empty_like(S_t)
        rsd.stepper_stokesian_dev(ctx, tab, c0.clone(), radii_t, 0.0, args.dt, [L, L, L], 1.0, mu, 1e-10, Um, Sm,
                                  precision=rsd.PREC_MIXED)
        Up, Sp = torch.empty_like(U_t), torch.empty_like(S_t)
        rsd.stepper_stokesian_dev(ctx, tab, c0.clone(), radii_t, 0.0, args.dt, [L, L, L], 1.0, mu, 1e-10, Up, Sp,
                                  precision=rsd.PREC_FP64)  # warm-up of the plain path's buffers
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        rsd.stepper_stokesian_dev(ctx, tab, c0.clone(), radii_t, 0.0, args.dt, [L, L, L], 1.0, mu, 1e-10, Up, Sp,
                                  precision=rsd.PREC_FP64)
        p1.record(stream)
        torch.cuda.synchronize(dev)
        pms = p0.elapsed_time(p1)
        pph = ctx.phase_ms()
        verr = float((Um - Up).abs().max() / Up.abs().max())
        serr = float((Sm - Sp).abs().max() / Sp.abs().max())
        plain = {"steps_per_s": 1000.0 / pms, "ms_per_step": pms,
                 "phases_ms": {"assembly": pph[0], "lub": pph[1], "solve": pph[2]},
                 "solve_tflops_fp64": solve_flops(N, "fp64") / (pph[2] * 1e-3) / 1e12,
                 "mixed_over_plain": (1000.0 / pms and value / ws / (1000.0 / pms)),
                 "vel_err_mixed_vs_fp64": verr, "stresslet_err_mixed_vs_fp64": serr}
    if rank != 0:
        if ws > 1:
            dist.barrier()
        return
    peaks = measured_peaks()
    fp64_peak = None if args.no_peaks else fp64_gemm_peak(torch, dev)
    fp32_peak = None if args.no_peaks else fp32_gemm_peak(torch, dev)
    NR, NI = infos[0][0], infos[0][1]
    ph = phases / args.steps
    asm_flop = ewald_flops(N, NR, NI)
    asm_rate = asm_flop / (ph[0] * 1e-3) / 1e12
    factor_ms = ph[2] - ph[3]
    solve_rate = solve_flops(N, args.precision) / (factor_ms * 1e-3) / 1e12
    dominant = "solve" if ph[2] >= ph[0] else "assembly"
    if dominant == "solve":
        rate, pk = solve_rate, (fp64_peak if args.precision == "fp64" else fp32_peak)
        pipe = "FP64" if args.precision == "fp64" else "FP32"
        pipe = "FP64" if args.precision == "fp64" else "TF32 tensor"
        src = ("cuBLAS %s 8192^3 measured in this run (the measured-peaks file has BF16 and HBM only)"
               % ("DGEMM" if args.precision == "fp64" else "FP32 GEMM with TF32 tensor cores"))
    else:
        rate, pk, pipe = asm_rate, fp64_peak, "FP64"
        src = "cuBLAS DGEMM 8192^3 measured in this run (the measured-peaks file has BF16 and HBM only)"
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic.txt")
    if os.path.exists(tfile):
        for line in open(tfile):
            k, _, v = line.partition("=")
            if k.strip() == "%s_%s_bytes_per_launch" % (dominant, args.precision):
                traffic = float(v)
    kname = {"solve": "factorisations of the solve (%s): Cholesky, SPD inverse, Cholesky of RPP" % args.precision,
             "assembly": "grand-mobility assembly (%s)" % args.precision}[dominant]
    roofline = {"bound": "tensor", "pipe": pipe, "kernel": kname, "achieved": rate,
                "peak": pk, "unit": "TFLOP/s", "frac": (rate / pk) if pk else None, "traffic": traffic,
                "peak_source": src}
    cpu = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        sec, desc = cpu_step_sample(pos, radii, L, N, args.dt, threads)
        cpu = {"value": 1.0 / sec, "unit": "steps/s", "cores": threads, "kind": "port", "sample": desc}
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic (seeded sphere packing, no dataset)",
            "config": {"workload": "STEPPER_Stokesian step, N=%d phi=%.2f gap>=%g, shear 1, dt %g, Ewald 1e-10, lub on"
                                   % (N, args.phi, args.gmin, args.dt),
                       "precision": args.precision, "tensor_cores": args.tensor_cores, "NR": NR, "NI": NI,
                       "l2": "inputs larger than L2 (grand mobility %.2f GB)" % (8 * (11 * N) ** 2 / 1e9),
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "phases_ms": {"assembly": ph[0], "lub": ph[1], "solve": ph[2], "refinement": ph[3]},
            "plain_fp64": plain,
            "refinement": {"iterations": [i[2] for i in infos], "residual": [i[3] for i in infos]},
            "kernels": {"assembly_tflops": asm_rate, "solve_tflops": solve_rate,
                        "assembly_algorithmic_flop": asm_flop, "solve_algorithmic_flop": solve_flops(N, args.precision)},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clocks}
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()


if __name__ == "__main__":
    main()
