#!/usr/bin/env python
"""Benchmark: IMEX time-steps/s of one production-size shell on the GB300, plus the Newton-GMRES
steady-state solve that follows it.

Workload ("shell N_r=30 N_theta=256, plain FP64"): one axisymmetric shell, N_r=30 Chebyshev points
(nr=29 interior), N_theta=256 modes, d=2, Pr=1, Tau=0.01, Ra_T=8000, Ra_S=500, dt=5e-4, seeded Gaussian
coefficients of amplitude 1e-3*exp(-k/8)*exp(-n/4) (synthetic: the reference ships no data).
One bench step = 100 IMEX time steps (Main.py:255-283) of the shell; the metric counts time steps.
After the timed time-stepping the state is handed to Newton-GMRES(restart 50) with the dt=1 operators
until |F|_2 <= 1e-10, reported as "newton".

Arms:
  default            libsdd_gb300 (hand-written sm_103a kernels through the C ABI)
  --impl reference   the reference's algorithm on the host cores (the numpy oracle restating it; the
                     reference itself is Python that needs numba/h5py/matplotlib and cannot run on the
                     GPU machine), a bounded sample of the same workload.

Run:  python bench.py [--gpus N --steps K --warmup W]   (N>1: launched by torch.distributed.run, one
independent replica shell per rank, weak scaling, no collective on the data path).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(workload="shell N_r=30 N_theta=256 plain FP64 IMEX time-stepping + Newton-GMRES(50)",
                N_r=30, N_theta=256, d=2.0, Pr=1.0, Tau=0.01, Ra_T=8000.0, Ra_S=500.0, dt=5e-4,
                steps_per_bench_step=100, seed=1234)
METRIC = "time-steps/s"
UNIT = "time-steps/s"
L2_FLUSH_BYTES = 512 << 20


def algorithmic(M, nr):
    """Per IMEX step of one shell: FP64 flops and bytes of the reference's algorithm (the radial
    contractions, 12 real transforms of length P per radius at 2.5 P log2 P, the pointwise products and
    the theta recurrences; the state in and out plus the three Linv sets read once):
    flops = 21 M nr^2 + 12 nr 2.5 P log2 P + 11 nr P + 40 nr M, bytes = 48 M nr + 24 M nr^2.
    Chain kernel alone: flops 8 M nr^2, bytes 24 M nr^2 + 48 M nr."""
    import math
    P = 3 * M // 2
    step_flops = 21 * M * nr ** 2 + 12 * nr * 2.5 * P * math.log2(P) + 11 * nr * P + 40 * nr * M
    step_bytes = 48 * M * nr + 24 * M * nr ** 2
    chain_flops = 8 * M * nr ** 2
    chain_bytes = 24 * M * nr ** 2 + 48 * M * nr
    return step_flops, step_bytes, chain_flops, chain_bytes


def split_flops(M, nr, precision):
    """FP64 and FP32 algorithmic flops of one IMEX step of one shell.  Plain: everything FP64.  Mixed: the
    nonlinear term (the 11 M nr^2 of its radial contractions, the 12 transforms, the products) is FP32 and the
    linear part (A2_SINE 2 M nr^2, the chains 8 M nr^2, the 40 nr M pointwise terms) stays FP64."""
    import math
    P = 3 * M // 2
    nl = 11 * M * nr ** 2 + 12 * nr * 2.5 * P * math.log2(P) + 11 * nr * P
    lin = 10 * M * nr ** 2 + 40 * nr * M
    return (nl + lin, 0.0) if precision == "fp64" else (lin, nl)


def kernel_algorithmic(name, M, nr, nch, layout=3):
    """Algorithmic FP64 flops and bytes of ONE launch of a step kernel for one shell (one IMEX step),
    P = 3M/2 grid points, nch chunks per chain (chunked layouts 2 and 3), np = (nch-1)(nch-2)/2:
      k_chain         the chain steps: flops 8 M nr^2 (psi [A B] 2nr x nr, T and S Linv nr x nr per mode),
                      bytes 32 M nr^2 (those matrices) + 48 M nr (h in, f out); under layout 2 plus the
                      sequential carry run by the last chunk: (nch-2) carried matvecs per chain, flops
                      24 (nch-2) nr^2, bytes 96 (nch-2) nr^2
      k_chain_carry   layout 3: the np products per chain at once, flops 24 np nr^2, bytes 96 np nr^2
      k_mode_mv(h)    h = Linv g: flops 6 M nr^2, bytes 24 M nr^2 + 48 M nr
      k_mode_mv(fix)  f += G s: flops 8 M nr^2 (nch-1)/nch, bytes 32 M nr^2 (nch-1)/nch + 48 M nr
      k_fx_deriv      4 radial contractions: flops 8 M nr^2, bytes 56 M nr; under layout 3 (time steps) plus
                      the previous step's chain correction, the k_mode_mv(fix) terms below
      k_fx_grid       9 inverse transforms (2.5 P log2 P each): flops 22.5 nr P log2 P, bytes 56 M nr + 72 nr P
      k_fx_prod       products + 3 forward transforms: flops 7.5 nr P log2 P + 11 nr P, bytes 72 nr P + 32 M nr
      k_fx_rows       fused nonlinear term: flops 8 M nr^2 + 30 nr P log2 P + 11 nr P, bytes 56 M nr
      k_rhs           flops 4 M nr^2 + 40 nr M, bytes 80 M nr"""
    import math
    P = 3 * M // 2
    lg = math.log2(P)
    f = (nch - 1) / nch if nch > 0 else 0.0
    npr = (nch - 1) * (nch - 2) // 2 if nch > 2 else 0
    seq = max(nch - 2, 0) if layout == 2 else 0
    table = {
        "k_chain": (8 * M * nr ** 2 + 24 * seq * nr ** 2, 32 * M * nr ** 2 + 48 * M * nr + 96 * seq * nr ** 2),
        "k_chain_carry": (24 * npr * nr ** 2, 96 * npr * nr ** 2),
        "k_mode_mv(h)": (6 * M * nr ** 2, 24 * M * nr ** 2 + 48 * M * nr),
        "k_mode_mv(fix)": (8 * M * nr ** 2 * f, 32 * M * nr ** 2 * f + 48 * M * nr),
        "k_fx_deriv": (8 * M * nr ** 2 + (8 * M * nr ** 2 * f if layout == 3 else 0),
                       56 * M * nr + ((32 * M * nr ** 2 * f + 48 * M * nr) if layout == 3 else 0)),
        "k_fx_grid": (22.5 * nr * P * lg, 56 * M * nr + 72 * nr * P),
        "k_fx_prod": (7.5 * nr * P * lg + 11 * nr * P, 72 * nr * P + 32 * M * nr),
        "k_fx_rows": (8 * M * nr ** 2 + 30 * nr * P * lg + 11 * nr * P, 56 * M * nr),
        "k_rhs": (4 * M * nr ** 2 + 40 * nr * M, 80 * M * nr),
    }
    return table[name]


# ------------------------------------------------------------------------------------------------
# clocks
# ------------------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock / throttle-reason samples every 200 ms while the timed region runs."""
    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []
        self.window = None      # (t0, t1) wall-clock bounds of the timed region (mark())

    def mark(self, t0, t1):
        """The timed region: samples stamped inside it (with a margin of one sampling period) are kept."""
        self.window = (t0, t1)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        import datetime
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = []
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                ts = None
            try:
                rows.append((ts, float(f[2]), float(f[3]), [nm for nm, v in zip(names, f[6:10])
                                                          if v.lower() == "active"]))
            except ValueError:
                continue
        inside = rows
        if self.window and rows:
            t0, t1 = self.window
            inside = [r for r in rows if r[0] is not None and t0 - 0.1 <= r[0] <= t1 + 0.1] or rows
        sm = sorted(r[1] for r in inside)
        smax = [r[2] for r in inside]
        reasons = sorted({nm for r in inside for nm in r[3]})
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(sm), "samples_in_timed_region": len(inside) if inside is not rows else None}


# ------------------------------------------------------------------------------------------------
# CPU baseline (the oracle), run in a child process so its BLAS/OpenMP threads are pinned at start-up
# ------------------------------------------------------------------------------------------------
def cpu_worker(seconds, threads, steps_per_sample, count=0):
    """Times IMEX steps of the workload with the oracle, in samples of steps_per_sample steps: `count`
    samples when count > 0, else samples until `seconds` have passed; prints one JSON line."""
    import numpy as np
    from oracle import sdd_oracle as O
    w = WORKLOAD
    M, N_r = w["N_theta"], w["N_r"]
    ops = O.Operators(M, N_r, w["d"], w["dt"], w["Pr"], w["Tau"])
    X = O.seeded_state(M, N_r - 1, w["seed"])
    X = O.step(ops, X, w["Ra_T"], w["Ra_S"], False)    # warm-up
    n = 0
    samples = []
    t_start = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        for _ in range(steps_per_sample):
            X = O.step(ops, X, w["Ra_T"], w["Ra_S"], False)
        samples.append(time.perf_counter() - t0)
        n += steps_per_sample
        if (count > 0 and len(samples) >= count) or (count <= 0 and time.perf_counter() - t_start >= seconds):
            break
    total = sum(samples)
    print(json.dumps({"steps": n, "seconds": total, "samples": samples, "threads": threads,
                      "finite": bool(np.isfinite(X).all())}))


def run_cpu_baseline(seconds=12.0, threads=1, steps_per_sample=5, count=0):
    env = dict(os.environ)
    for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS", "NUMEXPR_NUM_THREADS"):
        env[v] = str(threads)
    env["CUDA_VISIBLE_DEVICES"] = ""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--cpu-worker", str(seconds), str(threads),
           str(steps_per_sample), str(count)]
    out = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=600)
    if out.returncode != 0:
        raise RuntimeError("cpu baseline failed: " + out.stderr[-2000:])
    return json.loads(out.stdout.strip().splitlines()[-1])


# ------------------------------------------------------------------------------------------------
# distributed helpers
# ------------------------------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws, device):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------------------------------------
# reference arm
# ------------------------------------------------------------------------------------------------
def bench_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    # one bench step = the GPU arm's bench step (steps_per_bench_step IMEX steps of the shell) with all host
    # threads available to BLAS; exactly W untimed then K timed samples
    per = WORKLOAD["steps_per_bench_step"]
    r = run_cpu_baseline(threads=threads, steps_per_sample=per, count=args.warmup + args.steps)
    samples = r["samples"]
    timed = samples[args.warmup:]
    tsec = sum(timed)
    nsteps = per * len(timed)
    value = nsteps / tsec
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": len(timed), "warmup": args.warmup,
            "ms_per_step": 1e3 * tsec / len(timed), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Gaussian coefficients)",
            "config": dict(WORKLOAD, parallelism="single shell", l2="n/a (host)"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{nsteps} IMEX steps of the workload ({per} per bench step) with the "
                                       "numpy oracle restating the reference (reference un-JIT'd: numba "
                                       "unavailable)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------------------------
# batched workload: 64 shells of uneven (N_r, N_theta) and Ra_T, one captured graph per launch
# ------------------------------------------------------------------------------------------------
def bench_batched(device, precision, steps=1000, steps_per_launch=10, n_shells=64, fp64_peak=None):
    import numpy as np
    import torch
    from spectraldoublediffusiveconvection_gb300.batch import ShellBatch, config4_shells
    shells = config4_shells(n_shells, seed=1234)
    kw = dict(d=2.0, dt=1e-3, Pr=1.0, Tau=0.01, Ra_s=500.0, precision=precision, device=device)
    # tune on a scratch batch, run a fresh one with its choices (see ShellBatch.apply_tuning)
    tuning = ShellBatch(shells, **kw).autotune(steps_per_launch=steps_per_launch, reps=2)
    torch.cuda.synchronize(device)
    b = ShellBatch(shells, tuning=tuning, **kw)
    b.capture(steps_per_launch)
    launches = max(1, steps // steps_per_launch)
    b.replay(1)
    torch.cuda.synchronize(device)
    stream = torch.cuda.current_stream(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.replay(launches)
    e1.record(stream)
    torch.cuda.synchronize(device)
    sec = e0.elapsed_time(e1) * 1e-3
    finite = all(np.isfinite(x).all() for x in b.states())
    shell_steps = n_shells * launches * steps_per_launch
    groups = sorted(((g.plan.N_r, g.plan.N_fm, len(g.idx)) for g in b.groups), reverse=True)
    nsteps = launches * steps_per_launch
    f64 = sum(split_flops(s["N_theta"], s["N_r"] - 1, precision)[0] for s in shells) * nsteps
    f32 = sum(split_flops(s["N_theta"], s["N_r"] - 1, precision)[1] for s in shells) * nsteps
    roof = {"bound": "fp64", "achieved": f64 / sec / 1e12, "peak": fp64_peak, "unit": "TFLOP/s",
            "frac": f64 / sec / 1e12 / fp64_peak if fp64_peak else None,
            "peak_source": "measured live (sdd_measure_fp64_peak FMA loop)",
            "fp32_tflops": f32 / sec / 1e12,
            "note": "algorithmic FP64 flops of all shells (the implicit solves, A2_SINE and the pointwise linear "
                    "terms; in plain FP64 also the nonlinear term) over the measured FP64 FMA peak"}
    tune = {k: [v["chain_layout"], v["fx_split"], v.get("chunk_length")] for k, v in tuning.items() if isinstance(v, dict)
            and "chain_layout" in v}
    return {"shell_steps_per_s": shell_steps / sec, "seconds": sec, "shells": n_shells,
            "steps_per_shell": nsteps, "precision": precision, "roofline": roof,
            "graph": f"{launches} launches of one CUDA graph, {steps_per_launch} steps of all groups each",
            "groups": [f"N_r={a} N_theta={c} x{n}" for a, c, n in groups],
            "tuning_chain_layout_fx_split_chunk_lengths": tune, "finite": finite}


def bench_batched_plain_alone(device, steps=100):
    """The plain FP64 path on the batched workload's shells one at a time (each shell's own plan, the
    automatic kernel choices of a single shell): shell-steps/s of the whole set stepped sequentially, the
    same-workload denominator of the batched forms."""
    import torch
    from spectraldoublediffusiveconvection_gb300.batch import config4_shells
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    from spectraldoublediffusiveconvection_gb300.seeds import seeded_state
    shells = config4_shells(64, seed=1234)
    plans, total = {}, 0.0
    stream = torch.cuda.current_stream(device)
    for i, sh in enumerate(shells):
        key = (sh["N_theta"], sh["N_r"])
        if key not in plans:
            plans[key] = Plan(sh["N_theta"], sh["N_r"], 2.0, 1e-3, 1.0, 0.01, device=device)
        p = plans[key]
        X = torch.from_numpy(seeded_state(sh["N_theta"], sh["N_r"] - 1, 1234 + i)).to(device).reshape(1, -1)
        Y = p.step(X, sh["Ra"], 500.0, nsteps=steps)          # warm-up (graphs, workspace)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        p.step(Y, sh["Ra"], 500.0, nsteps=steps, out=X)
        e1.record(stream)
        torch.cuda.synchronize(device)
        total += e0.elapsed_time(e1) * 1e-3
    for p in plans.values():
        p.close()
    return {"shell_steps_per_s": 64 * steps / total, "steps_per_shell": steps,
            "how": "each of the 64 shells alone on the plain FP64 path, %d steps, one after the other" % steps}


def _cpu_batch_worker(job):
    """One host process of the batched CPU baseline: IMEX steps of its shells of the 64-shell workload with
    the oracle, round robin, for `seconds`; returns (shell-steps, seconds)."""
    idx, seconds = job
    from oracle import sdd_oracle as O
    from spectraldoublediffusiveconvection_gb300.batch import config4_shells
    shells = config4_shells(64, seed=1234)
    ops, X = {}, {}
    for i in idx:
        s = shells[i]
        key = (s["N_theta"], s["N_r"])
        if key not in ops:
            ops[key] = O.Operators(s["N_theta"], s["N_r"], 2.0, 1e-3, 1.0, 0.01)
        X[i] = O.seeded_state(s["N_theta"], s["N_r"] - 1, 1234 + i)
    n = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        for i in idx:
            s = shells[i]
            X[i] = O.step(ops[(s["N_theta"], s["N_r"])], X[i], s["Ra"], 500.0, False)
            n += 1
    return n, time.perf_counter() - t0


def bench_batched_cpu(seconds=10.0):
    """The batched workload on the host: one oracle process per core (spawned, one BLAS thread each), the
    64 shells dealt round robin; shell-steps of all processes over the slowest process's time."""
    import multiprocessing as mp
    n = os.cpu_count() or 1
    env_keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS", "NUMEXPR_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in env_keys}
    for k in env_keys:
        os.environ[k] = "1"
    try:
        with mp.get_context("spawn").Pool(n) as pool:
            res = pool.map(_cpu_batch_worker, [(list(range(w, 64, n)), seconds) for w in range(n)])
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    steps = sum(r[0] for r in res)
    t = max(r[1] for r in res)
    return {"value": steps / t, "unit": "shell-steps/s", "cores": n, "kind": "port",
            "sample": f"{steps} IMEX steps of the 64 shells (FP64 numpy oracle restating the reference), "
                      f"{n} processes of one thread, {seconds:.0f} s each (reference un-JIT'd: numba unavailable)"}


# ------------------------------------------------------------------------------------------------
# served workload: Poisson arrivals of continuation steps and 500-step integrations
# ------------------------------------------------------------------------------------------------
SERVED_SHAPES = [(nr, m) for nr in (20, 28, 36, 48) for m in (64, 128, 256, 512)]


def _served_stats(srv, reqs, wall, rate, st0):
    """Throughput and latency of one served run: continuation (Newton-corrector) solves/s and integration
    time-steps/s counted separately, p50/p99 overall and per kind with the queue / device split."""
    import numpy as np
    from spectraldoublediffusiveconvection_gb300 import serve
    con = [r for r in reqs if r.kind == "continue"]
    itg = [r for r in reqs if r.kind == "integrate"]
    ok_con = [r for r in con if r.error is None and r.result["converged"] and r.result["residual"] <= 1e-10]
    ok_int = [r for r in itg if r.error is None and np.isfinite(r.result["X"]).all()]
    lat = serve.latency_report(reqs)
    # FP64 work done: the integrations' IMEX steps (mixed form: the linear part and the chains in FP64) and
    # the continuation solves' Jacobian products (the FP64 chains, 8 M nr^2 per product and shell)
    f64 = sum(r.n_steps * split_flops(r.N_theta, r.N_r - 1, "mixed")[0] for r in ok_int)
    f64 += sum(r.result["matvecs"] * 8 * r.N_theta * (r.N_r - 1) ** 2 for r in ok_con)
    return {"offered_rate_per_s": rate, "requests": len(reqs), "wall_s": wall, "fp64_flops": f64,
            "continuation_solves_per_s": len(ok_con) / wall,
            "integration_steps_per_s": sum(r.n_steps for r in ok_int) / wall,
            "integration_requests_per_s": len(ok_int) / wall,
            "p50_ms": lat.get("p50_ms"), "p99_ms": lat.get("p99_ms"),
            "queue_p50_ms": lat.get("queue_p50_ms"), "queue_p99_ms": lat.get("queue_p99_ms"),
            "device_p50_ms": lat.get("device_p50_ms"), "device_p99_ms": lat.get("device_p99_ms"),
            "continuation": dict(serve.latency_report(con), n=len(con), converged_le_1e10=len(ok_con),
                                 max_residual=max((r.result["residual"] for r in con if r.result), default=None),
                                 mean_corrector_iters=float(np.mean([r.result["corrector_iters"] for r in con
                                                                     if r.result])) if ok_con else None),
            "integration": dict(serve.latency_report(itg), n=len(itg), finite=len(ok_int)),
            "errors": sum(r.error is not None for r in reqs),
            "error_samples": sorted({"%s %dx%d: %s" % (r.kind, r.N_r, r.N_theta, r.error) for r in reqs if r.error})[:5],
            "batching": {k: srv.stats[k] - st0[k] for k in srv.stats}}


P99_BOUND_MS = 1000.0


def bench_served(device, n_requests=1000, rate=200.0, seed=2024, frac_continue=0.7, con_workers=4, branch=None,
                 sweep=(100.0, 150.0, 200.0, 250.0, 275.0, 300.0, 400.0), sweep_requests=600, fp64_peak=None,
                 **server_kw):
    """The served mix at `rate` arrivals/s (the headline block), then an arrival-rate sweep on the same
    server: capacity = the highest swept rate whose p99 latency stays under P99_BOUND_MS over a run of
    `sweep_requests` requests (past saturation the queue, and with it p99, grows with the run), and the
    continuation solves with FP32 right-hand sides and an FP64 Krylov basis (mixed_matvec 2, the server's
    default) against an FP32 basis (3)."""
    import torch
    from spectraldoublediffusiveconvection_gb300 import serve
    t0 = time.perf_counter()
    if branch is None:
        branch = serve.branch_states(SERVED_SHAPES, Ra=9000.0, d=2.0, Pr=1.0, Tau=1.0, Ra_s=500.0, device=device)
    t_branch = time.perf_counter() - t0
    shapes = [s for s in SERVED_SHAPES if s in branch]
    server_kw.setdefault("con_mixed", 2)
    srv = serve.Server(d=2.0, Pr=1.0, Tau=1.0, Ra_s=500.0, dt=1e-3, device=device, con_workers=con_workers,
                       **server_kw).start()
    try:
        # warm-up: one request of each kind and shape builds the plans and workspaces
        for mv in (2, 3):
            srv.con_mixed = mv
            for sh in shapes:
                srv.submit(serve.Request("continue", sh[0], sh[1], 9000.0, X=branch[sh][0], sign=1.0, ds=50.0))
                srv.submit(serve.Request("integrate", sh[0], sh[1], 9000.0, n_steps=50, seed=1))
            srv.drain()
        srv.con_mixed = server_kw["con_mixed"]
        torch.cuda.synchronize(device)

        def run(r, n, sd, mv):
            srv.con_mixed = mv
            wl = serve.poisson_workload(n, r, shapes, branch, frac_continue=frac_continue, n_steps=500,
                                        ds=50.0, seed=sd)
            st0 = dict(srv.stats)
            wall = serve.run_workload(srv, wl)
            return _served_stats(srv, [q for _, q in wl], wall, r, st0)

        main = run(rate, n_requests, seed, server_kw["con_mixed"])
        curve = [run(r, sweep_requests, seed + 1 + i, server_kw["con_mixed"]) for i, r in enumerate(sweep)]
        other = 2 if server_kw["con_mixed"] == 3 else 3
        cmp_run = run(rate, sweep_requests, seed + 99, other)
        same = run(rate, sweep_requests, seed + 99, server_kw["con_mixed"])
    finally:
        srv.stop()
    # plans whose tensor-core kernel gave up waiting for its products (outputs NaN: such requests fail)
    tc_timeouts = sum(1 for p_ in srv._plans.values() if getattr(p_, "tensor_cores", False) and p_.tensor_core_timed_out())
    # the plain FP64 path on the same request mix: a sample of the continuation requests, each solved alone
    # (one shell, FP64 plan and FP64 Jacobian products), one after the other
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    import torch
    rng = __import__("numpy").random.default_rng(7)
    sample = [shapes[int(i)] for i in rng.integers(len(shapes), size=24)]
    plans = {}
    for sh in sorted(set(sample)):
        plans[sh] = Plan(sh[1], sh[0], 2.0, 1.0, 1.0, 1.0, device=device)
        Xw = torch.from_numpy(branch[sh][0].copy()).to(device).reshape(1, -1)
        plans[sh].contin_step(Xw, torch.tensor([9000.0], dtype=torch.float64, device=device), 500.0, 1.0, 50.0,
                              tangent_rtol=1e-4)                       # warm-up: workspace and first launch
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    n_ok = 0
    for k, sh in enumerate(sample):
        Xw = torch.from_numpy(branch[sh][0].copy()).to(device).reshape(1, -1)
        Rw = torch.tensor([9000.0], dtype=torch.float64, device=device)
        _, rr = plans[sh].contin_step(Xw, Rw, 500.0, 1.0 if k % 2 else -1.0, 50.0, tangent_rtol=1e-4)
        n_ok += int(rr[0]["converged"])
    torch.cuda.synchronize(device)
    plain_rate = len(sample) / (time.perf_counter() - t0)
    for p_ in plans.values():
        p_.close()
    # ... and a sample of the mix's integrations (500 steps of dt=1e-3 from seeded states), each alone on an
    # FP64 plan, so that the whole request mix has a plain-path rate: requests/s = 1 / (0.7 t_con + 0.3 t_int)
    from spectraldoublediffusiveconvection_gb300.seeds import seeded_state
    isample = [shapes[int(i)] for i in rng.integers(len(shapes), size=8)]
    iplans = {sh: Plan(sh[1], sh[0], 2.0, 1e-3, 1.0, 1.0, device=device) for sh in sorted(set(isample))}
    for sh, p_ in iplans.items():                                      # warm-up: workspace and step graphs
        p_.step(torch.from_numpy(seeded_state(sh[1], sh[0] - 1, 1)).to(device).reshape(1, -1), 9000.0, 500.0,
                nsteps=20)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    for k, sh in enumerate(isample):
        Xi = torch.from_numpy(seeded_state(sh[1], sh[0] - 1, 100 + k)).to(device).reshape(1, -1)
        iplans[sh].step(Xi, float(rng.uniform(8500.0, 9500.0)), 500.0, nsteps=500)
    torch.cuda.synchronize(device)
    t_int = (time.perf_counter() - t0) / len(isample)
    for p_ in iplans.values():
        p_.close()
    plain_mix = 1.0 / (frac_continue / plain_rate + (1.0 - frac_continue) * t_int)
    ok = [c for c in curve if c["p99_ms"] is not None and c["p99_ms"] <= P99_BOUND_MS]
    cap = max(ok, key=lambda c: c["offered_rate_per_s"]) if ok else None
    def roof(run):
        a = run["fp64_flops"] / run["wall_s"] / 1e12
        return {"bound": "fp64", "achieved": a, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": a / fp64_peak if fp64_peak else None,
                "note": "FP64 flops of the integrations' steps (linear part and chains of the mixed form) and of "
                        "the continuation products' chains (8 M nr^2 per product), over the run's wall time"}
    main.update({
        "roofline": roof(main), "capacity_roofline": roof(cap) if cap else None,
        "capacity_solves_per_s": cap["continuation_solves_per_s"] if cap else None,
        "capacity_offered_rate_per_s": cap["offered_rate_per_s"] if cap else None,
        "capacity_p50_ms": cap["p50_ms"] if cap else None, "capacity_p99_ms": cap["p99_ms"] if cap else None,
        "capacity_rule": "highest swept arrival rate with p99 <= %.0f ms over %d requests" % (P99_BOUND_MS,
                                                                                              sweep_requests),
        "plain_same_workload": {"continuation_solves_per_s": plain_rate, "sample": len(sample), "converged": n_ok,
                                "how": "24 continuation requests of the mix, each alone on an FP64 plan with FP64 "
                                       "Jacobian products, one after the other"},
        "capacity_vs_plain_same_workload": (cap["continuation_solves_per_s"] / plain_rate) if cap else None,
        "capacity_requests_per_s": (cap["continuation_solves_per_s"] + cap["integration_requests_per_s"]) if cap else None,
        "plain_same_mix": {"requests_per_s": plain_mix, "integration_seconds_per_request": t_int,
                           "continuation_seconds_per_request": 1.0 / plain_rate,
                           "how": "the mix's two kinds on the plain FP64 path one request at a time: 24 continuation "
                                  "requests and 8 of its 500-step integrations, combined 70/30 as the mix"},
        "capacity_vs_plain_same_mix": ((cap["continuation_solves_per_s"] + cap["integration_requests_per_s"])
                                       / plain_mix) if cap else None,
        "saturation_vs_plain_same_workload": max(c["continuation_solves_per_s"] for c in curve) / plain_rate,
        "sweep": [{k: c[k] for k in ("offered_rate_per_s", "continuation_solves_per_s", "integration_requests_per_s",
                                      "integration_steps_per_s",
                                      "p50_ms", "p99_ms", "queue_p99_ms", "device_p99_ms", "errors", "error_samples")}
                  for c in curve],
        "tensor_core_timeouts": tc_timeouts,
        "continuation_matvec_compare": {
            "mixed_matvec_%d" % server_kw["con_mixed"]: {k: same[k] for k in ("continuation_solves_per_s", "p50_ms",
                                                                            "p99_ms")},
            "mixed_matvec_%d" % other: {k: cmp_run[k] for k in ("continuation_solves_per_s", "p50_ms", "p99_ms")},
            "same_workload": "%d requests at %.0f/s" % (sweep_requests, rate)},
        "shapes": [f"{a}x{b}" for a, b in shapes], "branch_seconds": t_branch,
        "precision": {"integration": srv.int_precision + " (FP32 nonlinear term, FP64 implicit solves)",
                      "continuation": "mixed_matvec %d inside the Jacobian products, FP64 residual <= 1e-10"
                                      % server_kw["con_mixed"]},
        "chain_layout": srv.chain_layout, "tangent_rtol": srv.tangent_rtol, "con_workers": con_workers,
        "workload": "Poisson arrivals; 70% pseudo-arclength steps (ds=50, sign +-1) from steady states at "
                    "Ra_T=9000 on the Tau=1 branch, 30% 500-step integrations (dt=1e-3, Ra_T~U[8500,9500]) from "
                    "seeded states; N_r in {20,28,36,48}, N_theta in {64,128,256,512}; Ra_S=500, Pr=1, d=2"})
    return main


# ------------------------------------------------------------------------------------------------
# GB300 arm
# ------------------------------------------------------------------------------------------------
def bench_gb300(args):
    import numpy as np
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    device = torch.device("cuda", local if ws > 1 else 0)
    torch.cuda.set_device(device)

    import __graft_entry__
    __graft_entry__.build()
    from spectraldoublediffusiveconvection_gb300 import _lib
    from spectraldoublediffusiveconvection_gb300.seeds import seeded_state
    from spectraldoublediffusiveconvection_gb300.plan import Plan

    w = WORKLOAD
    M, N_r, nr = w["N_theta"], w["N_r"], w["N_r"] - 1
    chunk = w["steps_per_bench_step"]
    plan = Plan(M, N_r, w["d"], w["dt"], w["Pr"], w["Tau"], device=device)
    X0 = seeded_state(M, nr, w["seed"] + rank)
    Ra = torch.full((1,), w["Ra_T"], dtype=torch.float64, device=device)
    Ras = torch.full((1,), w["Ra_S"], dtype=torch.float64, device=device)
    Xa = torch.from_numpy(X0).to(device).reshape(1, -1)
    Xb = torch.empty_like(Xa)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream(device)

    # clocks sampled from before the warm-up (nvidia-smi takes a moment to start), kept for the timed region
    clocks = ClockSampler(device.index or 0)
    clocks.start()
    # warm-up
    for _ in range(args.warmup):
        plan.step(Xa, Ra, Ras, nsteps=chunk, out=Xb)
        Xa, Xb = Xb, Xa
    torch.cuda.synchronize()

    # ---- timed region (device-resident): K bench steps, L2 flushed between them (outside the events) --
    barrier(ws)
    torch.cuda.synchronize()
    wall0 = time.time()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        flush.zero_()
        evs[i][0].record(stream)
        plan.step(Xa, Ra, Ras, nsteps=chunk, out=Xb)
        evs[i][1].record(stream)
        Xa, Xb = Xb, Xa
    torch.cuda.synchronize()
    barrier(ws)
    clocks.mark(wall0, time.time())
    time.sleep(0.15)                  # one more sampling period past the region
    ms_total = sum(a.elapsed_time(b) for a, b in evs)
    ck = clocks.stop()
    ms_total = max_over_ranks(ms_total, ws, device)
    X_after = Xa.clone()
    time_steps = args.steps * chunk * ws
    value = time_steps / (ms_total * 1e-3)

    # ---- e2e through the public API with host buffers (pinned), copies inside the timed region ----
    h_in = torch.from_numpy(X0.copy()).reshape(1, -1).pin_memory()
    h_out = torch.empty_like(h_in).pin_memory()
    d_in = torch.empty_like(Xa)
    d_out = torch.empty_like(Xa)
    for _ in range(max(1, args.warmup)):
        d_in.copy_(h_in, non_blocking=True)
        plan.step(d_in, Ra, Ras, nsteps=chunk, out=d_out)
        h_out.copy_(d_out, non_blocking=True)
        torch.cuda.synchronize()
    barrier(ws)
    e2e_s = 0.0
    for i in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d_in.copy_(h_in, non_blocking=True)
        plan.step(d_in, Ra, Ras, nsteps=chunk, out=d_out)
        h_out.copy_(d_out, non_blocking=True)
        torch.cuda.synchronize()
        e2e_s += time.perf_counter() - t0
        h_in, h_out = h_out, h_in
    barrier(ws)
    e2e_s = max_over_ranks(e2e_s, ws, device)
    e2e_value = time_steps / e2e_s
    nbytes = X0.size * 8

    # ---- per-kernel durations: a CUDA event after every kernel launch of each step (launched one by one) --
    nprof = min(200, args.steps * chunk)
    kp = plan.kernel_profile(X_after, Ra, Ras, nprof)
    n_kp = sum(v[1] for v in kp.values())
    ms3, _ = plan.step_profile(X_after, Ra, Ras, nprof)
    ms3 = [m / nprof for m in ms3]
    kavg = {k: v[0] / v[1] for k, v in kp.items()}                 # ms per launch
    kstep = {k: v[0] / nprof for k, v in kp.items()}               # ms per step
    dom = max(kstep, key=kstep.get)
    step_flops, step_bytes, chain_flops, chain_bytes = algorithmic(M, nr)
    fp64 = __import__("ctypes").c_double(0.0)
    _lib.check(_lib.lib().sdd_measure_fp64_peak(__import__("ctypes").byref(fp64),
                                                 __import__("ctypes").c_void_p(stream.cuda_stream)),
               "sdd_measure_fp64_peak")
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    hbm_src = "of measured" if "hbm_gbs" in peaks else "of fallback"
    traffic = None
    try:
        tr = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
        traffic = tr.get(dom)
    except (OSError, ValueError):
        pass
    lay, _, nch_used = plan.chain_choice(1)
    kflops, kbytes = kernel_algorithmic(dom, M, nr, nch_used, lay)
    dom_s = kavg[dom] * 1e-3
    achieved_gbs = kbytes / dom_s / 1e9
    fp64_peak_tf = fp64.value / 1e3
    # FP64 arithmetic, not HBM, is what bounds this path (a dependent chain of FP64 operations over a few
    # thousand unknowns per shell): the primary fraction is algorithmic FP64 flops over the measured FP64 peak
    roofline = {"bound": "fp64", "achieved": kflops / dom_s / 1e12, "peak": fp64_peak_tf, "unit": "TFLOP/s",
                "frac": kflops / dom_s / 1e12 / fp64_peak_tf, "traffic": traffic, "kernel": dom,
                "peak_source": "measured live (sdd_measure_fp64_peak FMA loop over all SMs)",
                "algorithmic_flops_per_launch": kflops, "launch_ms": kavg[dom],
                "hbm": {"achieved_gbs": achieved_gbs, "peak_gbs": hbm_peak, "frac": achieved_gbs / hbm_peak,
                        "peak_source": hbm_src, "algorithmic_bytes_per_launch": kbytes},
                "kernel_ms_per_step": kstep,
                "stage_ms_per_step": dict(zip(["nonlinear_term", "rhs", "implicit_solves"], ms3)),
                "step_fp64_tflops": step_flops / (ms_total * 1e-3 / (args.steps * chunk)) / 1e12,
                "step_fp64_frac": step_flops / (ms_total * 1e-3 / (args.steps * chunk)) / 1e12 / fp64_peak_tf}

    # ---- Newton-GMRES(50) from the state after the time stepping --------------------------------------
    newton = None
    if not args.no_newton:
        plan1 = Plan(M, N_r, w["d"], 1.0, w["Pr"], w["Tau"], device=device)
        Xn = X_after.clone()
        plan1.newton(Xn.clone(), Ra, Ras, tol=1e-10, restart=50, max_newton=2)   # warm-up (allocations)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = plan1.newton(Xn, Ra, Ras, tol=1e-10, restart=50, gmres_rtol=1e-4, max_newton=20)[0]
        torch.cuda.synchronize()
        tn = time.perf_counter() - t0
        newton = {"solves_per_s": 1.0 / tn, "seconds": tn, "newton_iters": res["newton_iters"],
                  "matvecs": res["matvecs"], "residual0": res["residual0"], "residual": res["residual"],
                  "converged": res["converged"], "tol": 1e-10, "restart": 50}
        # batched: 64 shells of the same shape in one sdd_newton_gmres call (each shell its own Krylov
        # space), FP32 nonlinear term, right-hand sides and h matvecs inside the Jacobian products and an FP32
        # Krylov basis (mixed_matvec 3; FP64 chains, residual and update), FP64 residual <= 1e-10; the same
        # with an FP64 basis (mixed_matvec 2) beside it
        nb = 64
        planm = Plan(M, N_r, w["d"], 1.0, w["Pr"], w["Tau"], precision="mixed", device=device)
        planm.set_chain_layout(4)      # whole chains, split rows: measured best for the 64-shell Newton batch
        pert = torch.from_numpy(np.stack([seeded_state(M, N_r - 1, 500 + i) for i in range(nb)])).to(device)
        Xb0 = X_after.reshape(1, -1) + pert
        Rab = torch.linspace(7000.0, 9000.0, nb, dtype=torch.float64, device=device)
        tbm = {}
        for mvb in (2, 3):
            planm.newton(Xb0.clone(), Rab, Ras, tol=1e-10, restart=50, max_newton=1, mixed_matvec=mvb)  # warm-up
            Xb = Xb0.clone()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rb = planm.newton(Xb, Rab, Ras, tol=1e-10, restart=50, gmres_rtol=1e-4, max_newton=20, mixed_matvec=mvb)
            torch.cuda.synchronize()
            tbm[mvb] = (time.perf_counter() - t0, rb)
        tb, rb = tbm[3]
        rb2 = tbm[2][1]
        # the plain FP64 path on the same problems: a sample of 8 of the 64 shells solved one at a time with
        # FP64 Jacobian products (the single-shell automatic kernel choices)
        sample = list(range(0, nb, nb // 8))
        Xs = Xb0[sample].clone()
        plan1.newton(Xs[0:1].clone(), Rab[0:1], Ras, tol=1e-10, restart=50, max_newton=1)      # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rp = [plan1.newton(Xs[i:i + 1], Rab[sample[i]:sample[i] + 1], Ras, tol=1e-10, restart=50, gmres_rtol=1e-4,
                           max_newton=20)[0] for i in range(len(sample))]
        torch.cuda.synchronize()
        tp = time.perf_counter() - t0
        # per Jacobian product and shell: the FP64 chains (8 M nr^2; the FP32 basis's Gram-Schmidt runs in FP32
        # and is not counted); every shell counted for every product (the count of the slowest shell: an
        # upper bound on the work done)
        f64_b = nb * rb[0]["matvecs"] * (8 * M * nr ** 2)
        newton["batched"] = {"solves_per_s": nb / tb, "seconds": tb, "shells": nb, "mixed_matvec": 3,
                             "fp64_basis": {"mixed_matvec": 2, "solves_per_s": nb / tbm[2][0],
                                            "converged": sum(r["converged"] for r in rb2),
                                            "max_residual": max(r["residual"] for r in rb2),
                                            "matvecs": rb2[0]["matvecs"]},
                             "converged": sum(r["converged"] for r in rb),
                             "max_residual": max(r["residual"] for r in rb), "matvecs": rb[0]["matvecs"],
                             "vs_plain_single_shell": (nb / tb) / (1.0 / tn),
                             "plain_same_workload": {"solves_per_s": len(sample) / tp, "shells": len(sample),
                                                     "converged": sum(r["converged"] for r in rp),
                                                     "matvecs_mean": sum(r["matvecs"] for r in rp) / len(rp),
                                                     "how": "8 of the 64 problems, one at a time, FP64 plan "
                                                            "and FP64 Jacobian products"},
                             "vs_plain_same_workload": (nb / tb) / (len(sample) / tp),
                             "roofline": {"bound": "fp64", "achieved": f64_b / tb / 1e12, "peak": fp64_peak_tf,
                                          "unit": "TFLOP/s", "frac": f64_b / tb / 1e12 / fp64_peak_tf,
                                          "note": "FP64 chain flops of every product of every shell (upper "
                                                  "bound) over the measured FP64 FMA peak; the Gram-Schmidt "
                                                  "work of the FP32 basis is FP32"},
                             "workload": "64 shells N_r=30 N_theta=256, Ra_T 7000..9000, Tau=0.01, from the "
                                         "time-stepped state plus seeded perturbations"}

    # ---- mixed precision on the same shell: FP32 nonlinear term, FP64 solves ---------------------------
    mixed = None
    if not args.no_newton:
        pm = Plan(M, N_r, w["d"], w["dt"], w["Pr"], w["Tau"], precision="mixed", device=device)
        Xm_a = torch.from_numpy(X0).to(device).reshape(1, -1)
        Xm_b = torch.empty_like(Xm_a)
        for _ in range(args.warmup):
            pm.step(Xm_a, Ra, Ras, nsteps=chunk, out=Xm_b)
        torch.cuda.synchronize()
        evm = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        for i in range(args.steps):
            flush.zero_()
            evm[i][0].record(stream)
            pm.step(Xm_a, Ra, Ras, nsteps=chunk, out=Xm_b)
            evm[i][1].record(stream)
            Xm_a, Xm_b = Xm_b, Xm_a
        torch.cuda.synchronize()
        mixed_rate = args.steps * chunk / (sum(a.elapsed_time(b) for a, b in evm) * 1e-3)
        # trajectory to t = 5 (10^4 steps of dt = 5e-4) from the seeded state, against the FP64 path
        nt = int(round(5.0 / w["dt"]))
        Xs = torch.from_numpy(X0).to(device).reshape(1, -1)
        Xmix = pm.step(Xs, Ra, Ras, nsteps=nt)
        Xd64 = plan.step(Xs, Ra, Ras, nsteps=nt)
        err = float(torch.linalg.vector_norm(Xmix - Xd64) / torch.linalg.vector_norm(Xd64))
        pmn = Plan(M, N_r, w["d"], 1.0, w["Pr"], w["Tau"], precision="mixed", device=device)
        pmn.newton(X_after.clone(), Ra, Ras, tol=1e-10, restart=50, max_newton=1, mixed_matvec=True)  # warm-up
        Xn_m = X_after.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rm = pmn.newton(Xn_m, Ra, Ras, tol=1e-10, restart=50, gmres_rtol=1e-4, max_newton=20, mixed_matvec=True)[0]
        torch.cuda.synchronize()
        tm = time.perf_counter() - t0
        mixed = {"time_steps_per_s": mixed_rate, "vs_fp64_single_shell": mixed_rate / (value / ws),
                 "trajectory_rel_err_t5_vs_fp64": err, "t5_steps": nt,
                 "newton_residual": rm["residual"], "newton_converged": rm["converged"],
                 "newton_matvecs": rm["matvecs"], "newton_solves_per_s": 1.0 / tm,
                 "newton_start": "the FP64 time-stepped state (as the FP64 Newton above)",
                 "workload": "the same shell, FP32 nonlinear term (transforms, products, radial derivatives), "
                             "FP64 right-hand sides, implicit solves, Newton residual and GMRES; the FP64 path "
                             "it is compared with matches the oracle to 1e-12 per step"}

    batched = None
    if not args.no_batched:
        import numpy as np  # noqa: F401
        bm = bench_batched(device, "mixed", fp64_peak=fp64_peak_tf)
        bd = bench_batched(device, "fp64", fp64_peak=fp64_peak_tf)
        plain = value / ws
        alone = bench_batched_plain_alone(device)
        batched = {"mixed": bm, "fp64": bd,
                   "mixed_vs_plain_single_shell": bm["shell_steps_per_s"] / plain,
                   "fp64_vs_plain_single_shell": bd["shell_steps_per_s"] / plain,
                   "plain_same_shells_alone": alone,
                   "mixed_vs_plain_same_shells": bm["shell_steps_per_s"] / alone["shell_steps_per_s"],
                   "cpu_baseline": None if args.no_cpu else bench_batched_cpu(),
                   "workload": "64 shells, N_r in {20,24,30,36}, N_theta in {64,128,256,384}, Ra_T ~ U[6000,12000],"
                               " Ra_S=500, Pr=1, Tau=0.01, dt=1e-3, 1000 steps each (seed 1234)"}

    served = None
    if rank == 0 and not args.no_served:
        served = bench_served(device, n_requests=args.served_requests, fp64_peak=fp64_peak_tf)

    cpu = None
    if rank == 0 and not args.no_cpu:
        r = run_cpu_baseline(seconds=args.cpu_seconds, threads=1, steps_per_sample=5)
        cpu = {"value": r["steps"] / r["seconds"], "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{r['steps']} IMEX steps of the same shell with the numpy oracle restating the "
                         "reference, 1 thread (reference un-JIT'd: numba unavailable)"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_total / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded Gaussian coefficients, amplitude 1e-3 exp(-k/8) exp(-n/4))",
                "config": dict(WORKLOAD, parallelism=f"replicas x{ws}" if ws > 1 else "single shell",
                               l2="flushed between timed bench steps (512 MiB write)"),
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nbytes,
                        "d2h_bytes_per_step": nbytes,
                        "api": "Plan.step on a pinned host state copied in/out every bench step"},
                # per bench step: the kernels of `chunk` steps, plus the one deferred chain correction that a
                # multi-step call applies at its end (the profile's launches over nprof steps include it once)
                "gpu_launches": args.steps * (chunk * (n_kp // nprof) + n_kp % nprof),
                "roofline": roofline, "cpu_baseline": cpu, "clocks": ck, "mixed": mixed,
                "batched": batched, "served": served,
                # last, so that a reader of the line's tail sees the Newton solves/s (plain and batched)
                "newton": newton}
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def profile_newton_batch(mixed_matvec=2):
    """One Newton iteration (residual, one GMRES(50) solve, update) of the 64-shell batched Newton workload
    inside an NVTX range "newton_batched", for a kernel launch list of the batched Jacobian products:
    ncu --nvtx --nvtx-include "newton_batched/" ... python bench.py --profile-newton-batch [MODE].  The start:
    the seeded shell after 2000 IMEX steps of dt=5e-4 plus the 64 seeded perturbations of the bench workload;
    MODE the mixed_matvec value (2: FP64 Krylov basis, 3: FP32 basis)."""
    import numpy as np
    import torch
    from spectraldoublediffusiveconvection_gb300.seeds import seeded_state
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    w = WORKLOAD
    M, N_r = w["N_theta"], w["N_r"]
    device = torch.device("cuda", 0)
    p = Plan(M, N_r, w["d"], w["dt"], w["Pr"], w["Tau"], device=device)
    X0 = torch.from_numpy(seeded_state(M, N_r - 1, w["seed"])).to(device).reshape(1, -1)
    Xa = p.step(X0, w["Ra_T"], w["Ra_S"], nsteps=2000)
    nb = 64
    pert = torch.from_numpy(np.stack([seeded_state(M, N_r - 1, 500 + i) for i in range(nb)])).to(device)
    Xb0 = Xa.reshape(1, -1) + pert
    Rab = torch.linspace(7000.0, 9000.0, nb, dtype=torch.float64, device=device)
    Ras = torch.full((nb,), w["Ra_S"], dtype=torch.float64, device=device)
    q = Plan(M, N_r, w["d"], 1.0, w["Pr"], w["Tau"], precision="mixed", device=device)
    q.set_chain_layout(4)
    q.newton(Xb0.clone(), Rab, Ras, tol=1e-10, restart=50, max_newton=1, mixed_matvec=mixed_matvec)   # warm-up
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("newton_batched")
    r = q.newton(Xb0.clone(), Rab, Ras, tol=1e-10, restart=50, max_newton=1, mixed_matvec=mixed_matvec)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    print(json.dumps({"profile": "newton_batched", "shells": nb, "mixed_matvec": mixed_matvec,
                      "jacobian_products": r[0]["matvecs"]}))
    return 0


def profile_deriv_tc(batch):
    """k_deriv_tc alone (the mixed form's 3xTF32 radial contractions) on `batch` FP32 shells of N_r=30,
    N_theta=256: three warm-up launches, then ten timed with CUDA events.  For
    ncu --set full -k regex:k_deriv_tc -s 3 -c 1 ... python bench.py --profile-deriv-tc <batch>."""
    import torch
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    M, N_r = 256, 30
    nr = N_r - 1
    device = torch.device("cuda", 0)
    p = Plan(M, N_r, 2.0, 5e-4, 1.0, 0.01, precision="mixed", device=device)
    g = torch.Generator(device="cpu").manual_seed(1)
    X = torch.randn((batch, p.n_state), generator=g, dtype=torch.float32).to(device)
    out = torch.empty((batch, 4, nr, M), dtype=torch.float32, device=device)
    for _ in range(3):
        p.deriv_tc(X, out)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        p.deriv_tc(X, out)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 10
    io = batch * (3 * M * nr + 4 * nr * M) * 4
    print(json.dumps({"profile": "deriv_tc", "shells": batch, "ms_per_launch": ms, "algorithmic_bytes": io,
                      "GB_per_s": io / ms / 1e6, "timed_out": p.tensor_core_timed_out()}))
    return 0


def profile_step_batch(precision, layout, batch=64, steps=1):
    """The kernels of `steps` IMEX steps of `batch` shells N_r=30, N_theta=256 sharing one plan (dt=1e-3,
    Ra_T 6000..12000, seeded states 1000+i), launched one by one with an event after each kernel
    (Plan.kernel_profile) after two warm-up steps; chain layout `layout` (0 automatic), the fused row kernel.
    For ncu launch lists and per-kernel captures of the batched time step:
    ncu ... -k regex:<kernel> -c 1 ... python bench.py --profile-step-batch <precision> <layout>."""
    import numpy as np
    import torch
    from spectraldoublediffusiveconvection_gb300.seeds import seeded_state
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    M, N_r = 256, 30
    device = torch.device("cuda", 0)
    p = Plan(M, N_r, 2.0, 1e-3, 1.0, 0.01, precision=precision, device=device)
    p.set_chain_layout(layout)
    p.set_fx_split(1)
    X = torch.from_numpy(np.stack([seeded_state(M, N_r - 1, 1000 + i) for i in range(batch)])).to(device)
    Ra = torch.linspace(6000.0, 12000.0, batch, dtype=torch.float64, device=device)
    X = p.step(X, Ra, 500.0, nsteps=2)
    torch.cuda.synchronize()
    prof = p.kernel_profile(X, Ra, 500.0, steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    p.step(X, Ra, 500.0, nsteps=20)
    e1.record()
    torch.cuda.synchronize()
    print(json.dumps({"profile": "step_batch", "precision": precision, "shells": batch,
                      "chain_layout": p.chain_choice(batch)[0], "graph_ms_per_step": e0.elapsed_time(e1) / 20,
                      "kernels_ms": {k: v[0] / steps for k, v in prof.items()}}))
    return 0


def profile_uneven_batch(precision):
    """One launch (10 steps of every shape group) of the batched workload's captured graph (64 shells, N_r in
    {20,24,30,36}, N_theta in {64,128,256,384}, the default per-group choices) inside an NVTX range
    "uneven_batch", after two warm-up launches, for a kernel launch list of the batched time step:
    ncu --nvtx --nvtx-include "uneven_batch/" ... python bench.py --profile-uneven-batch <precision>."""
    import torch
    from spectraldoublediffusiveconvection_gb300.batch import ShellBatch, config4_shells
    device = torch.device("cuda", 0)
    b = ShellBatch(config4_shells(64, seed=1234), d=2.0, dt=1e-3, Pr=1.0, Tau=0.01, Ra_s=500.0,
                   precision=precision, device=device)
    b.capture(10)
    b.replay(2)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("uneven_batch")
    e0.record()
    b.replay(1)
    e1.record()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    groups = [(g.plan.N_r, g.plan.N_fm, len(g.idx), g.plan.chain_choice(len(g.idx))[0]) for g in b.groups]
    print(json.dumps({"profile": "uneven_batch", "precision": precision, "ms_per_launch": e0.elapsed_time(e1),
                      "groups_Nr_Ntheta_shells_layout": groups}))
    return 0


def probe_phase_boundaries():
    """The cost of a phase boundary inside a captured CUDA graph (a kernel boundary) against a grid-wide
    barrier inside one persistent cooperative kernel (sdd_probe_phase_boundaries): 64 phases over one CTA
    per SM (the single-shell step's kernels fill at most about one SM each) and over four CTAs per SM,
    without work (the boundary alone) and with 256 dependent FP64 multiply-adds per thread per phase."""
    import ctypes
    import torch
    from spectraldoublediffusiveconvection_gb300 import _lib
    device = torch.device("cuda", 0)
    torch.cuda.set_device(device)
    L = _lib.lib()
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    stream = ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
    out = []
    for ctas in (sms, 4 * sms):
        for work in (0, 256):
            g, pz, to = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_int(0)
            nph = 64
            _lib.check(L.sdd_probe_phase_boundaries(ctas, 256, nph, work, 5, ctypes.byref(g), ctypes.byref(pz),
                                                    ctypes.byref(to), stream), "sdd_probe_phase_boundaries")
            out.append({"ctas": ctas, "threads": 256, "phases": nph, "fp64_fma_per_thread_per_phase": work,
                        "graph_us": g.value, "persistent_us": pz.value,
                        "graph_us_per_phase": g.value / nph, "persistent_us_per_phase": pz.value / nph,
                        "barrier_timed_out": bool(to.value)})
    print(json.dumps({"probe": "phase_boundaries", "results": out}))
    return 0


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "--cpu-worker":
        cpu_worker(float(sys.argv[2]), int(sys.argv[3]), int(sys.argv[4]),
                   int(sys.argv[5]) if len(sys.argv) > 5 else 0)
        return 0
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-newton", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--served-requests", type=int, default=1000)
    ap.add_argument("--profile-newton-batch", nargs="?", type=int, const=2, default=None, metavar="MODE")
    ap.add_argument("--profile-deriv-tc", type=int, metavar="SHELLS")
    ap.add_argument("--profile-step-batch", nargs=2, metavar=("PRECISION", "LAYOUT"))
    ap.add_argument("--profile-uneven-batch", metavar="PRECISION")
    ap.add_argument("--probe-phase-boundaries", action="store_true")
    args = ap.parse_args()
    if args.probe_phase_boundaries:
        return probe_phase_boundaries()
    if args.profile_newton_batch is not None:
        return profile_newton_batch(args.profile_newton_batch)
    if args.profile_deriv_tc:
        return profile_deriv_tc(args.profile_deriv_tc)
    if args.profile_step_batch:
        return profile_step_batch(args.profile_step_batch[0], int(args.profile_step_batch[1]))
    if args.profile_uneven_batch:
        return profile_uneven_batch(args.profile_uneven_batch)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return bench_reference(args)
    return bench_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
