#!/usr/bin/env python
"""Throughput of the hydrodynamic step (steps/s) on one GB300.

Workload: N = 2048 monodisperse spheres, volume fraction 0.5, seeded minimum
gap 1e-4 a, Lees-Edwards shear rate 1, dt = 5e-4, Ewald tolerance 1e-10,
lubrication on -- one STEPPER_Stokesian step per timed iteration, all inputs
resident in HBM.  The grand mobility alone (4.06 GB FP64) is larger than L2,
so no flush is needed between iterations.

The step's cost follows the Lees-Edwards strain: CALC_LATTICE_INVERSE
(csd_post.f90:158-183) gives NR = NI = 3 at zero skew and up to 5 near skew
1, i.e. 685 to 2661 Ewald images per pair (1538 on average over a strain
cycle).  The headline therefore runs the step at a stratified set of
strains covering one cycle -- skew (k + 1/2)/S, k = 0..S-1 (S = 5: 0.1, 0.3,
0.5, 0.7, 0.9; NR = NI = 3, 4, 4, 4, 5; 1543 images per pair on average) --
each from a configuration valid at that strain (configs.sheared_series: the
seeded packing sheared affinely with the lattice and its overlaps relaxed),
the timed steps spread round-robin over the strata, and `value` is the
strain-averaged steps/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision mixed|fp64] [--strata 5] [--N 2048] [--phi 0.5]

Prints one JSON line (rank 0).  With --gpus N > 1 under torchrun every rank
steps its own independent replica (the step does not shard; replicas only).
--impl reference times the CPU restatement of the reference's routines on the
host cores instead (bounded samples per step, extrapolated; see CpuModel).
--mode long runs the 10,000-step long run through the driver's time loop,
--mode ensemble the ensemble of 256 uneven replicas (replica-steps/s), and
--mode learned the learned preconditioner's PCG solves on the N = 1000
near-contact workload.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "steps/s N=2048 φ=0.5: mixed+learned vs plain FP64 on GB300, vel err ≤1e-8"
SEED_BASE = 20260000


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--strata", type=int, default=5, help="strains of the Lees-Edwards cycle the steps run at")
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
    ap.add_argument("--real-passes", type=int, default=0, choices=[0, 1, 2, 3, 4],
                    help="mixed real-space sum: passes over the near images (0: the library's default)")
    ap.add_argument("--factor-schedule", type=int, default=1, choices=[0, 1],
                    help="mixed form's FP32 Cholesky: 1 look-ahead on the diagonal chain, 0 in-order panels")
    ap.add_argument("--validate-cpu-model", action="store_true",
                    help="(reference arm) time one whole CPU step at N=512 and compare it with the sample model")
    ap.add_argument("--refinement", default="stationary", choices=["gmres", "stationary"],
                    help="mixed form's FP64 refinement: flexible GMRES or the stationary iteration")
    ap.add_argument("--mode", default="cycle", choices=["cycle", "long", "ensemble", "learned"],
                    help="cycle: the strain-stratified headline; long: the 10,000-step run through the driver; "
                         "ensemble: 256 uneven replicas; learned: the learned preconditioner's PCG solves")
    ap.add_argument("--replicas", type=int, default=256, help="(ensemble) number of replicas")
    ap.add_argument("--ens-steps", type=int, default=50, help="(ensemble) steps of every replica")
    ap.add_argument("--workers", type=int, default=16, help="(ensemble) concurrent contexts")
    ap.add_argument("--long-steps", type=int, default=10000)
    ap.add_argument("--plain-steps", type=int, default=5, help="(long) plain FP64 steps beside the mixed run")
    ap.add_argument("--long-seconds", type=float, default=0.0, help="(long) wall-time budget; 0: none")
    ap.add_argument("--contact", type=float, default=1000.0,
                    help="(long) host contact repulsion F0 in units of 6 pi mu a^2 gammadot (0: none)")
    ap.add_argument("--contact-range", type=float, default=0.01, help="(long) its decay length, in radii")
    ap.add_argument("--out-dir", default=None, help="(long) where yeta_mu.txt and the viscosity series go")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_seed(rank):
    """Seed of rank `rank`'s packing: every replica steps its own system."""
    return SEED_BASE + 5000 + rank


def strata_skews(S):
    """Skews (k + 1/2)/S of the strain cycle, k = 0..S-1."""
    return [(k + 0.5) / S for k in range(S)]


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
            d = json.load(fp)
            d["source"] = "measured"
            return d
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


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


def gemm_peak(torch, dev, dtype, tf32=False):
    """cuBLAS GEMM rate on this GPU (TFLOP/s), 8192^3, best of a few: the
    builder-measured denominators for the FP64 form (DGEMM) and for the
    mixed form's TF32 factorisations (FP32 GEMM with TF32 tensor cores),
    beside the measured BF16 peak."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = tf32
    n = 8192
    a = torch.randn(n, n, dtype=dtype, device=dev)
    b = torch.randn(n, n, dtype=dtype, device=dev)
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


def images(NR, NI):
    return (2 * NR + 1) ** 3, (2 * NI + 1) ** 3 - 1


def ewald_flops(N, NR, NI):
    """Algorithmic FLOP of one grand-mobility assembly: 500 per real image and
    150 per reciprocal vector of the reference's cubes, over the unordered
    pairs (all images) and the self terms (n != 0 and k != 0)."""
    nr, nk = images(NR, NI)
    pairs = N * (N - 1) // 2
    return pairs * (nr * 500.0 + nk * 150.0) + N * ((nr - 1) * 500.0 + nk * 150.0)


SOLVE_FLOP_PER_N3 = 1403.0  # Cholesky + SPD inverse of M (n = 11N) and Cholesky of RPP (6N)


def lattice_of(skew, L, radii, ews=1e-10):
    """NR, NI of CALC_LATTICE_INVERSE at skew `skew` (the oracle's lattice
    routines, host only)."""
    from oracle import oracle as o
    lat = o.set_lattice_skew(skew, [L, L, L], 1.0)
    o.calc_lattice_inverse(lat, ews, radii)
    return lat.NR, lat.NI


# ---------------------------------------------------------------- CPU arm
class CpuModel:
    """Seconds per step of the CPU restatement of the reference's routines
    (the oracle: C + scipy's OpenBLAS LAPACK) at the full workload, from
    bounded samples timed each step and scaled by unit counts:
      assembly  PER_GRPERY_INV_FRI on the first 96 particles of the stratum's
                configuration in the full box at its strain (the same images
                per pair), scaled to N(N-1)/2 pairs plus N self terms;
      lub       lubmxcalc on a 512-particle box at the same volume fraction,
                scaled by (N/512)^2 (pair sweep and dense outputs are O(N^2));
      solve     LAPACK DPOTRF + DPOTRI of an assembled 512-particle grand
                mobility (n = 5632, the oracle's own matrix at phi) plus
                DPOTRF of its 6N RPP block, scaled by (N/512)^3."""

    def __init__(self, N, phi, gmin, strata, L, radii, sweeps, threads):
        from oracle import oracle as o
        self.o = o
        self.N, self.strata, self.L, self.radii, self.threads = N, strata, L, radii, threads
        self.mu = o.mu_f_dimensionless(1.0)
        self.tab = o.LubTab(os.path.join(ROOT, "tests", "golden", "lubdat"))
        cfg = _configs()
        self.ns = min(512, N)
        self.pos_s, _, self.Ls = cfg.packing(self.ns, phi, gmin, SEED_BASE + 5900, sweeps=min(sweeps, 50))
        self.radii_s = np.ones(self.ns)
        lat = o.set_lattice_skew(0.0, [self.Ls] * 3, 1.0)
        t0 = time.perf_counter()
        G, _ = o.per_grpery_inv_fri(self.pos_s, self.radii_s, lat, 1e-10, self.mu)
        self.setup_assembly_s = time.perf_counter() - t0
        self.Ms = np.asfortranarray(G)
        self.Rs = np.asfortranarray(np.linalg.inv(G)[:6 * self.ns, :6 * self.ns] + np.eye(6 * self.ns))

    def sample(self, k):
        """One bounded sample at stratum k; returns (seconds per full step,
        dict of measured sample seconds and scale factors)."""
        from scipy.linalg import lapack
        o, N = self.o, self.N
        pos, skew = self.strata[k]
        lat = o.set_lattice_skew(skew, [self.L] * 3, 1.0)
        na = min(96, N)
        t0 = time.perf_counter()
        o.per_grpery_inv_fri(pos[:na], self.radii[:na], lat, 1e-10, self.mu)
        t_asm = time.perf_counter() - t0
        s_asm = (N * (N - 1) / 2 + N) / (na * (na - 1) / 2 + na)
        lat2 = o.set_lattice_skew(0.0, [self.Ls] * 3, 1.0)
        t0 = time.perf_counter()
        o.lubmxcalc(self.pos_s, self.radii_s, lat2, self.mu, self.tab)
        t_lub = time.perf_counter() - t0
        s_lub = (N / self.ns) ** 2
        A = self.Ms.copy(order="F")
        B = self.Rs.copy(order="F")
        t0 = time.perf_counter()
        c, _ = lapack.dpotrf(A, lower=0, clean=0, overwrite_a=1)
        lapack.dpotri(c, lower=0, overwrite_c=1)
        lapack.dpotrf(B, lower=0, clean=0, overwrite_a=1)
        t_sol = time.perf_counter() - t0
        s_sol = (N / self.ns) ** 3
        NR, NI = lat.NR, lat.NI
        total = t_asm * s_asm + t_lub * s_lub + t_sol * s_sol
        return total, {"skew": skew, "NR": NR, "NI": NI, "assembly_sample_s": t_asm, "assembly_scale": s_asm,
                       "lub_sample_s": t_lub, "lub_scale": s_lub, "solve_sample_s": t_sol, "solve_scale": s_sol}

    def describe(self, k):
        return ("port (C restatement + OpenBLAS LAPACK), %d threads; per step, at the step's stratum of the strain "
                "cycle: assembly of %d particles' pairs at that strain scaled to %d pairs, lub at N=%d scaled by "
                "N^2, DPOTRF+DPOTRI of an assembled n=%d grand mobility + DPOTRF of its RPP scaled by n^3 "
                "(extrapolated from samples timed every step)" % (self.threads, min(96, self.N),
                                                                  self.N * (self.N - 1) // 2, self.ns, 11 * self.ns))


def validate_cpu_model(args, threads):
    """One whole oracle step at N = 512 (phi, gap and strain 0 as the model's
    samples) against the model's prediction for N = 512."""
    from oracle import oracle as o
    cfg = _configs()
    N = 512
    pos, radii, L = cfg.packing(N, args.phi, args.gmin, SEED_BASE + 5901, sweeps=50)
    model = CpuModel(N, args.phi, args.gmin, [(pos, 0.0)], L, radii, 50, threads)
    pred, parts = model.sample(0)
    tab = o.LubTab(os.path.join(ROOT, "tests", "golden", "lubdat"))
    t0 = time.perf_counter()
    o.stepper_stokesian(pos, radii, [L, L, L], 0.0, args.dt, 1.0, o.mu_f_dimensionless(1.0), 1e-10, tab)
    full = time.perf_counter() - t0
    return {"N": N, "full_step_s": full, "model_s": pred, "model_over_full": pred / full, "parts": parts}


def reference_arm(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    from oracle import oracle as o
    o.build()
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    cfg = _configs()
    skews = strata_skews(max(1, args.strata))
    series, radii, L = cfg.sheared_series(args.N, args.phi, args.gmin, replica_seed(0), skews, sweeps=args.sweeps)
    strata = list(zip(series, skews))
    model = CpuModel(args.N, args.phi, args.gmin, strata, L, radii, args.sweeps, threads)
    S = len(strata)
    for w in range(args.warmup):
        model.sample((S - 1 - w) % S)
    ts, parts = [], []
    for k in range(args.steps):
        t, p = model.sample(k % S)
        ts.append(t)
        parts.append(p)
    sec = float(np.mean(ts))
    v = 1.0 / sec
    line = {"metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded sphere packing sheared to each stratum)",
            "config": {"workload": workload_name(args), "strata_skew": skews, "l2": "inputs larger than L2"},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "steps/s", "cores": threads, "kind": "port",
                             "sample": model.describe(0), "extrapolated": True, "samples": parts},
            "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if args.validate_cpu_model:
        line["cpu_model_check"] = validate_cpu_model(args, threads)
    print(json.dumps(line), flush=True)


def _configs():
    import importlib.util
    path = os.path.join(ROOT, "regularized-stokesian-dynamics_gb300", "configs.py")
    spec = importlib.util.spec_from_file_location("rsd_configs_only", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def workload_name(args):
    return ("STEPPER_Stokesian step, N=%d phi=%.2f gap>=%g, shear 1, dt %g, Ewald 1e-10, lub on; strain-averaged "
            "over %d strata of the Lees-Edwards cycle" % (args.N, args.phi, args.gmin, args.dt, args.strata))


def read_traffic(key):
    tfile = os.path.join(ROOT, "profiles", "traffic.txt")
    if os.path.exists(tfile):
        for line in open(tfile):
            k, _, v = line.partition("=")
            if k.strip() == key:
                try:
                    return float(v.split()[0])
                except (ValueError, IndexError):
                    return None
    return None


# ---------------------------------------------------------------- long run
def periodic_fts_control(path, dt, steps, k_write, linerr=1e-10):
    """The reference's example control_file.dat switched to the periodic FTS
    case with lubrication at shear rate 1 (records as INIT_READ_CONTROL reads
    them, initial_conf.f90:109-189)."""
    src = open(os.path.join(ROOT, "tests", "golden", "io", "control_file.dat")).read().split("\n")
    end = (steps - 1) * dt  # main.f90 leaves the loop once T > END_TIME: `steps` steps
    rec = {1: ".true.", 3: ".true.", 7: ".false.", 9: ".true.", 10: ".true.", 18: "1.0", 19: "1.0", 20: "0.0",
           27: "1.0", 33: repr(linerr), 36: "0.0", 37: repr(end), 38: repr(dt), 39: str(k_write)}
    for i, v in rec.items():
        src[i] = v + "    ! periodic FTS case with lubrication, shear rate 1"
    with open(path, "w") as fp:
        fp.write("\n".join(src))


def long_run(args):
    """The long dense run: N = 2048, phi = 0.5, gap >= 1e-4 a, shear rate 1,
    dt = 5e-4, --long-steps steps (10,000: strain 5, five Lees-Edwards
    cycles) through the driver's time loop (driver.py, main.f90's loop and
    files) on the fused mixed-precision step; the relative viscosity of every
    step is kept (yeta_mu.txt holds every K_WRITE-th, as main.f90 writes it).
    The plain FP64 form runs its own first --plain-steps steps from the same
    start for the viscosity difference."""
    import tempfile

    import torch

    import __graft_entry__ as ge
    rsd = ge.load_package()
    out = args.out_dir or tempfile.mkdtemp(prefix="rsd_long_")
    os.makedirs(out, exist_ok=True)
    work = tempfile.mkdtemp(prefix="rsd_long_work_")
    N, dt = args.N, args.dt
    pos, radii, L = rsd.configs.packing(N, args.phi, args.gmin, replica_seed(0), sweeps=args.sweeps)
    control, init = os.path.join(work, "control_file.dat"), os.path.join(work, "initial_config.dat")
    periodic_fts_control(control, dt, args.long_steps, 100)
    rsd.driver_files.write_initial_config(init, pos, radii, [L, L, L])
    ctx = rsd.Context(0)
    ctx.set_tensor_cores(args.tensor_cores)
    tab = rsd.LubTab(rsd.lubdat_dir())
    series = []
    fp64_steps = []
    mixed = rsd.driver_step(ctx, tab, rsd.PREC_MIXED, fp64_fallback=True,
                            on_fallback=lambda T, why: fp64_steps.append((T, why)))

    soft = rsd.contact.SoftContact(N, L, f0=args.contact, delta=args.contact_range) if args.contact > 0 else None

    class _Stop(Exception):
        pass

    def step(conf, r, T, dt_, LB, gamma, mu_f, ews, Fe=None):
        if args.long_seconds > 0 and time.perf_counter() - t0 > args.long_seconds:
            raise _Stop("wall-time budget of %.0f s reached" % args.long_seconds)
        n64 = len(fp64_steps)
        o = mixed(conf, r, T, dt_, LB, gamma, mu_f, ews, Fe=Fe)
        i = o["info"]
        # 0: mixed; 1: mixed, finished by flexible GMRES; 2: taken in FP64
        how = 2 if len(fp64_steps) > n64 else int(i.fallback)
        gap = soft.min_gap if soft is not None else float("nan")
        series.append((T, float(o["yeta_mu"][0]), i.NR, i.NI, i.iterations, i.residual, how, gap))
        return o

    import signal

    def _on_term(signum, frame):  # a time limit ends the run: report how far it got
        raise _Stop("stopped by signal %d" % signum)

    old_term = signal.signal(signal.SIGTERM, _on_term)
    t0 = time.perf_counter()
    err = None
    try:
        res = rsd.driver.run(control, init, step, os.path.join(work, "output.VTF"), os.path.join(out, "yeta_mu.txt"),
                             forces=soft.forces if soft is not None else None,
                             max_steps=args.long_steps)
    except (Exception, _Stop) as e:  # report how far the run got
        err = "%s: %s" % (type(e).__name__, e)
        res = {"steps": len(series)}
    signal.signal(signal.SIGTERM, old_term)
    wall = time.perf_counter() - t0
    with open(os.path.join(out, "eta_r_series.csv"), "w") as fp:
        fp.write("# strain, relative viscosity, NR, NI, refinement iterations, residual, "
                 "solve (0 mixed, 1 mixed finished by flexible GMRES, 2 FP64), smallest surface gap\n")
        for T, y, nr, ni, it, rr, how, gap in series:
            fp.write("%.6f,%.12e,%d,%d,%d,%.3e,%d,%.4e\n" % (T, y, nr, ni, it, rr, how, gap))
    # plain FP64 beside the first steps, from the same start
    mu = rsd.mu_f_dimensionless(1.0)
    conf = pos.copy()
    plain = []
    d = rsd.driver_files.read_initial_config(init)
    conf = np.array(d["conf"])
    T = 0.0
    soft64 = rsd.contact.SoftContact(N, L, f0=args.contact, delta=args.contact_range) if args.contact > 0 else None
    for k in range(min(args.plain_steps, len(series))):
        Fe = soft64.forces(conf, T) if soft64 is not None else None
        o = rsd.STEPPER_Stokesian(ctx, tab, conf, radii, T, dt, [L, L, L], 1.0, mu, 1e-10, Fe=Fe,
                                  precision=rsd.PREC_FP64)
        plain.append(float(o["yeta_mu"][0]))
        conf, T = o["conf"], T + dt
    per_strain = []
    ys = np.array([s_[1] for s_ in series]) if series else np.zeros(0)
    ts = np.array([s_[0] for s_ in series]) if series else np.zeros(0)
    for c in range(int(math.ceil(ts.max() + 1e-12)) if len(ts) else 0):
        sel = (ts >= c) & (ts < c + 1)
        if sel.any():
            per_strain.append({"strain": [c, c + 1], "eta_r_mean": float(ys[sel].mean()),
                               "eta_r_std": float(ys[sel].std()), "steps": int(sel.sum())})
    its = [s_[4] for s_ in series]
    line = {"metric": "long run: steps/s N=%d phi=%.2f, %d steps through the driver" % (N, args.phi, args.long_steps),
            "value": len(series) / wall if wall > 0 else None, "unit": "steps/s", "steps": len(series),
            "wall_s": wall, "completed": err is None and len(series) == args.long_steps, "error": err,
            "precision": "mixed", "strain_end": float(ts.max()) if len(ts) else 0.0,
            "eta_r_per_strain_unit": per_strain,
            "refinement_iterations": {"mean": float(np.mean(its)) if its else None,
                                      "max": int(np.max(its)) if its else None},
            "gmres_finished_steps": int(sum(1 for s_ in series if s_[6] == 1)),
            "contact": ({"F0_over_6pi_mu_a2_gammadot": args.contact, "range_over_a": args.contact_range,
                         "smallest_gap": float(np.nanmin([s_[7] for s_ in series])) if series else None}
                        if soft is not None else None),
            "fp64_steps": len(fp64_steps), "fp64_steps_first": [[float(t), w] for t, w in fp64_steps[:10]],
            "NR_range": [int(min(s_[2] for s_ in series)), int(max(s_[2] for s_ in series))] if series else None,
            "plain_fp64_eta_r": plain, "mixed_eta_r_first": [s_[1] for s_ in series[:len(plain)]],
            "eta_r_rel_diff_first_steps": [abs(a - b) / abs(b) for a, b in zip([s_[1] for s_ in series], plain)],
            "files": {"yeta_mu": os.path.join(out, "yeta_mu.txt"), "series": os.path.join(out, "eta_r_series.csv")}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- ensemble
def _pack_replica(job):
    """One replica's packing (a top-level function, so that spawned worker
    processes can run it)."""
    N, phi, gmin, seed, sweeps = job
    return _configs().packing(N, phi, gmin, seed, sweeps=sweeps)


def ensemble_run(args):
    """The ensemble workload: --replicas replicas, N uniform in [32, 256], phi
    uniform in [0.10, 0.50], shear rate log-uniform in [0.1, 10], seeded
    minimum gap 1e-3 a, dt 1e-3, --ens-steps steps each, mixed precision;
    replica-steps/s over the whole ensemble (replicas on --workers
    concurrent contexts, largest first, kernel settings per size class from
    the autotuner)."""
    import __graft_entry__ as ge
    rsd = ge.load_package()
    ens_mod = rsd.ensemble
    specs = ens_mod.replica_specs(args.replicas, SEED_BASE + 3000)
    t0 = time.perf_counter()
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    jobs = [(s_["N"], s_["phi"], 1e-3, s_["seed"], min(args.sweeps, 30)) for s_ in specs]
    with ProcessPoolExecutor(mp_context=mp.get_context("spawn")) as ex:  # before any CUDA work
        packs = list(ex.map(_pack_replica, jobs, chunksize=4))
    t_pack = time.perf_counter() - t0
    ens = ens_mod.Ensemble(rsd, specs, packs, dt=1e-3, workers=args.workers)
    table = ens.autotune()
    lib = rsd.library()
    ens.run(1)  # warm-up: every context grows its buffers
    n0 = lib.rsd_launch_count()
    wall = ens.run(args.ens_steps)
    launches = lib.rsd_launch_count() - n0
    its = [i[2] for i in ens.info]
    res = [i[3] for i in ens.info]
    by_class = {}
    for k in range(len(ens_mod.SIZE_CLASSES)):
        members = [r for r, s_ in enumerate(specs) if ens_mod.size_class(s_["N"]) == k]
        if members:
            by_class[str(k)] = {"replicas": len(members), "N_range": ens_mod.SIZE_CLASSES[k],
                                "setting": table.get(str(k))}
    line = {"metric": "replica-steps/s, %d replicas N in [32,256], phi in [0.10,0.50], shear log-uniform [0.1,10]"
                      % args.replicas,
            "value": args.replicas * args.ens_steps / wall, "unit": "replica-steps/s", "higher_is_better": True,
            "steps_per_replica": args.ens_steps, "wall_s": wall, "workers": ens.workers, "precision": "mixed",
            "refinement_iterations": {"mean": float(np.mean(its)), "max": int(np.max(its))},
            "worst_residual": float(np.max(res)), "size_classes": by_class, "packing_s": t_pack,
            "gpu_launches": launches,
            "schedule": "replicas on concurrent contexts (one CUDA stream each), largest first; not one launch"}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- learned preconditioner
def learned_run(args):
    """The learned-preconditioner workload: N = 1000, phi = 0.5, a quarter of
    the spheres in near-contact pairs with gaps log-uniform in [1e-4, 1e-1] a
    (a seed not used in training), strain 0.25; RPP in FP64 (plain path);
    RPP x = b by PCG in FP64 to 1e-12 with each preconditioner: iterations,
    FP64 residual and time, beside a library Cholesky solve for scale."""
    import torch

    import __graft_entry__ as ge
    rsd = ge.load_package()
    N = 1000
    dev = torch.device("cuda", 0)
    series, radii, L = rsd.configs.sheared_series(N, 0.5, 1e-4, SEED_BASE + 4999, [0.25],
                                                  sweeps=min(args.sweeps, 100), near_contact=True)
    ctx = rsd.Context(0)
    tab = rsd.LubTab(rsd.lubdat_dir())
    mu = rsd.mu_f_dimensionless(1.0)
    conf_t = torch.tensor(series[0], dtype=torch.float64, device=dev)
    radii_t = torch.tensor(radii, dtype=torch.float64, device=dev)
    rpp, lat = rsd.resistance_pp_dev(ctx, tab, conf_t, radii_t, 0.25, [L, L, L], 1.0, mu, 1e-10)
    net = rsd.LearnedPreconditioner.trained(0)
    b = torch.tensor(np.random.default_rng(2).normal(size=6 * N), device=dev)
    out = {}
    for name, mode in (("none", rsd.PC_NONE), ("jacobi", rsd.PC_JACOBI), ("block_jacobi", rsd.PC_BLOCK_JACOBI),
                       ("fsai", rsd.PC_FSAI), ("learned", rsd.PC_LEARNED)):
        rsd.pcg_dev(ctx, net, mode, conf_t, radii_t, lat, rpp, b, tol=1e-12, maxit=20000)  # warm-up
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        x, it, res = rsd.pcg_dev(ctx, net, mode, conf_t, radii_t, lat, rpp, b, tol=1e-12, maxit=20000)
        rsd._sync_ctx(ctx)
        dt_ = time.perf_counter() - t0
        r = b - rpp @ x
        out[name] = {"iterations": it, "residual": res, "fp64_residual": float(r.norm() / b.norm()),
                     "seconds": dt_}
    A = rpp.contiguous().clone()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    Lc = torch.linalg.cholesky(A)
    xc = torch.cholesky_solve(b[:, None], Lc)[:, 0]
    torch.cuda.synchronize(dev)
    out["cholesky_library"] = {"seconds": time.perf_counter() - t0,
                               "fp64_residual": float((b - rpp @ xc).norm() / b.norm()),
                               "note": "torch (cuSOLVER) Cholesky, for scale only"}
    line = {"metric": "learned preconditioner, N=1000 phi=0.5 near-contact: PCG iterations to 1e-12 on RPP",
            "value": out["learned"]["iterations"], "unit": "iterations", "higher_is_better": False,
            "unpreconditioned_iterations": out["none"]["iterations"], "solves": out}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU arm
def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
        return
    if args.mode == "long":
        long_run(args)
        return
    if args.mode == "ensemble":
        ensemble_run(args)
        return
    if args.mode == "learned":
        learned_run(args)
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
    N = args.N
    S = max(1, args.strata)
    skews = strata_skews(S)
    series, radii, L = rsd.configs.sheared_series(N, args.phi, args.gmin, replica_seed(rank), skews,
                                                  sweeps=args.sweeps)
    mu = rsd.mu_f_dimensionless(1.0)
    ctx = rsd.Context(local)
    ctx.set_tensor_cores(args.tensor_cores)
    ctx.set_factor_schedule(args.factor_schedule)
    if args.real_passes:
        ctx.set_mixed_real_passes(args.real_passes)
    ctx.set_refinement(1 if args.refinement == "gmres" else 0)
    tab = rsd.LubTab(rsd.lubdat_dir())
    radii_t = torch.tensor(radii, dtype=torch.float64, device=dev)
    conf = [torch.tensor(p, dtype=torch.float64, device=dev) for p in series]
    Ts = list(skews)  # shear rate 1: strain = T
    U_t = torch.empty(6 * N, dtype=torch.float64, device=dev)
    S_t = torch.empty(5 * N, dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    stream = torch.cuda.ExternalStream(ctx.stream)
    lib = rsd.library()

    def step(k, precision=prec):
        y, info = rsd.stepper_stokesian_dev(ctx, tab, conf[k], radii_t, Ts[k], args.dt, [L, L, L], 1.0, mu, 1e-10,
                                            U_t, S_t, precision=precision)
        Ts[k] += args.dt
        return y, info

    # warm-up from the largest images down, so that every grow-only buffer
    # has its final size before the timed region
    for w in range(args.warmup):
        step((S - 1 - w) % S)
    sampler = ClockSampler(local) if rank == 0 else None
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    if sampler:
        sampler.start()
    n0 = lib.rsd_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    phases = np.zeros(4)
    infos, per_stratum = [], [[] for _ in range(S)]
    for i in range(args.steps):
        k = i % S
        y, info = step(k)
        ph = ctx.phase_ms()
        phases += ph
        infos.append((k, info.NR, info.NI, info.iterations, info.residual, float(y[0])))
        per_stratum[k].append(float(ph[:3].sum()))
    e1.record(stream)
    torch.cuda.synchronize(dev)
    launches = lib.rsd_launch_count() - n0
    ms = e0.elapsed_time(e1)
    clocks = sampler.stop() if sampler else None
    ms = max_over_ranks(ms, ws, dist, torch, dev)
    ms_per_step = ms / args.steps
    value = replica_throughput(ws, args.steps, ms * 1e-3)
    # end to end through the host C-ABI call (H2D of the inputs, D2H of the
    # results every step), round-robin over the same strata
    e2e = None
    if not args.no_e2e:
        conf_h = [c.cpu().numpy().copy() for c in conf]
        Te = list(Ts)
        t0 = time.perf_counter()
        for i in range(args.steps):
            k = i % S
            out = rsd.STEPPER_Stokesian(ctx, tab, conf_h[k], radii, Te[k], args.dt, [L, L, L], 1.0, mu, 1e-10,
                                        precision=prec)
            conf_h[k] = out["conf"]
            Te[k] += args.dt
        te = max_over_ranks(time.perf_counter() - t0, ws, dist, torch, dev)
        e2e = {"value": replica_throughput(ws, args.steps, te), "unit": "steps/s",
               "h2d_bytes_per_step": 8 * (3 * N + N), "d2h_bytes_per_step": 8 * (3 * N + 6 * N + 5 * N)}
    # the plain FP64 form at every stratum (its own step from the same
    # configuration): steps/s and the mixed form's errors against it
    plain = None
    if not args.no_plain and args.precision == "mixed":
        pms_all, verr, serr, yerr, pph_all = [], 0.0, 0.0, 0.0, np.zeros(4)
        for k in range(S):
            c0 = conf[k].clone()
            Um, Sm = torch.empty_like(U_t), torch.empty_like(S_t)
            ym, _ = rsd.stepper_stokesian_dev(ctx, tab, c0.clone(), radii_t, Ts[k], args.dt, [L, L, L], 1.0, mu,
                                              1e-10, Um, Sm, precision=rsd.PREC_MIXED)
            Up, Sp = torch.empty_like(U_t), torch.empty_like(S_t)
            if k == 0:  # the plain path's buffers, once
                rsd.stepper_stokesian_dev(ctx, tab, c0.clone(), radii_t, Ts[k], args.dt, [L, L, L], 1.0, mu, 1e-10,
                                          Up, Sp, precision=rsd.PREC_FP64)
            p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            p0.record(stream)
            yp, _ = rsd.stepper_stokesian_dev(ctx, tab, c0.clone(), radii_t, Ts[k], args.dt, [L, L, L], 1.0, mu,
                                              1e-10, Up, Sp, precision=rsd.PREC_FP64)
            p1.record(stream)
            torch.cuda.synchronize(dev)
            pms_all.append(p0.elapsed_time(p1))
            pph_all += ctx.phase_ms()
            verr = max(verr, float((Um - Up).abs().max() / Up.abs().max()))
            serr = max(serr, float((Sm - Sp).abs().max() / Sp.abs().max()))
            yerr = max(yerr, abs(ym[0] - yp[0]) / abs(yp[0]))
        pms = float(np.mean(pms_all))
        pph = pph_all / S
        plain = {"steps_per_s": 1000.0 / pms, "ms_per_step": pms, "ms_per_stratum": pms_all,
                 "phases_ms": {"assembly": pph[0], "lub": pph[1], "solve": pph[2]},
                 "solve_tflops_fp64": SOLVE_FLOP_PER_N3 * N ** 3 / (pph[2] * 1e-3) / 1e12,
                 "mixed_over_plain": (value / ws) / (1000.0 / pms),
                 "vel_err_mixed_vs_fp64": verr, "stresslet_err_mixed_vs_fp64": serr,
                 "viscosity_err_mixed_vs_fp64": yerr}
    if rank != 0:
        if ws > 1:
            dist.barrier()
        return
    peaks = measured_peaks()
    fp64_peak = None if args.no_peaks else gemm_peak(torch, dev, torch.float64)
    tf32_peak = None if args.no_peaks else gemm_peak(torch, dev, torch.float32, tf32=True)
    ph = phases / args.steps
    asm_flop = float(np.mean([ewald_flops(N, i[1], i[2]) for i in infos]))
    asm_rate = asm_flop / (ph[0] * 1e-3) / 1e12
    solve_flop = SOLVE_FLOP_PER_N3 * N ** 3
    solve_rate = solve_flop / (ph[2] * 1e-3) / 1e12
    bf16 = peaks.get("bf16_tflops")
    traffic = read_traffic("solve_%s_bytes_per_step" % args.precision)
    roofline = {"bound": "tensor", "kernel": "the step's solve phase (%s): the factorisations on tcgen05 and the FP64 "
                                             "refinement, %g N^3 FLOP per step" % (args.precision, SOLVE_FLOP_PER_N3),
                "achieved": solve_rate, "peak": bf16, "unit": "TFLOP/s",
                "frac": solve_rate / bf16 if bf16 else None, "traffic": traffic,
                "peak_source": "dense BF16 tensor rate, %s (MEASURED_PEAKS.json)" % peaks.get("source"),
                "tf32_peak_builder_measured": tf32_peak,
                "frac_of_tf32_builder_measured": solve_rate / tf32_peak if tf32_peak else None,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum over the solve phase's launches "
                                  "of one step (profiles/traffic.txt)"}
    by_stratum = []
    for k in range(S):
        its = [i for i in infos if i[0] == k]
        if not its:
            continue
        by_stratum.append({"skew": skews[k], "NR": its[0][1], "NI": its[0][2],
                           "images_per_pair": sum(images(its[0][1], its[0][2])),
                           "ms_per_step": float(np.mean(per_stratum[k])),
                           "iterations": [i[3] for i in its], "residual": [i[4] for i in its],
                           "yeta_mu": [i[5] for i in its]})
    cpu = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        model = CpuModel(N, args.phi, args.gmin, list(zip(series, skews)), L, radii, args.sweeps, threads)
        secs, parts = [], []
        for k in range(S):
            t, p = model.sample(k)
            secs.append(t)
            parts.append(p)
        cpu = {"value": 1.0 / float(np.mean(secs)), "unit": "steps/s", "cores": threads, "kind": "port",
               "sample": model.describe(0), "extrapolated": True, "samples": parts}
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic (seeded sphere packing sheared to each stratum, no dataset)",
            "config": {"workload": workload_name(args), "precision": args.precision,
                       "tensor_cores": args.tensor_cores, "factor_schedule": args.factor_schedule,
                       "refinement": args.refinement, "strata_skew": skews,
                       "mean_images_per_pair": float(np.mean([sum(images(i[1], i[2])) for i in infos])),
                       "l2": "inputs larger than L2 (grand mobility %.2f GB)" % (8 * (11 * N) ** 2 / 1e9),
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "phases_ms": {"assembly": ph[0], "lub": ph[1], "solve": ph[2], "refinement": ph[3]},
            "strata": by_stratum,
            "plain_fp64": plain,
            "kernels": {"assembly_tflops_algorithmic": asm_rate, "assembly_algorithmic_flop": asm_flop,
                        "solve_tflops_algorithmic": solve_rate, "solve_algorithmic_flop": solve_flop,
                        "fp64_dgemm_peak_builder_measured": fp64_peak},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clocks}
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()


if __name__ == "__main__":
    main()
