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
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
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
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


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
    # one bench step = a bounded sample of the workload: 5 IMEX steps with all host threads available to
    # BLAS; exactly W untimed then K timed samples
    per = 5
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
            "config": dict(WORKLOAD, steps_per_bench_step=per, l2="n/a (host)"),
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
def bench_batched(device, precision, steps=1000, steps_per_launch=10, n_shells=64):
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
    return {"shell_steps_per_s": shell_steps / sec, "seconds": sec, "shells": n_shells,
            "steps_per_shell": launches * steps_per_launch, "precision": precision,
            "graph": f"{launches} launches of one CUDA graph, {steps_per_launch} steps of all groups each",
            "groups": [f"N_r={a} N_theta={c} x{n}" for a, c, n in groups], "tuning": tuning, "finite": finite}


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


def bench_served(device, n_requests=1000, rate=200.0, seed=2024, frac_continue=0.7, con_workers=4, branch=None,
                 **server_kw):
    import numpy as np
    import torch
    from spectraldoublediffusiveconvection_gb300 import serve
    t0 = time.perf_counter()
    if branch is None:
        branch = serve.branch_states(SERVED_SHAPES, Ra=9000.0, d=2.0, Pr=1.0, Tau=1.0, Ra_s=500.0, device=device)
    t_branch = time.perf_counter() - t0
    shapes = [s for s in SERVED_SHAPES if s in branch]
    srv = serve.Server(d=2.0, Pr=1.0, Tau=1.0, Ra_s=500.0, dt=1e-3, device=device, con_workers=con_workers,
                       **server_kw).start()
    # warm-up: one request of each kind and shape builds the plans and workspaces
    warm = []
    for sh in shapes:
        warm.append(srv.submit(serve.Request("continue", sh[0], sh[1], 9000.0, X=branch[sh][0], sign=1.0, ds=50.0)))
        warm.append(srv.submit(serve.Request("integrate", sh[0], sh[1], 9000.0, n_steps=50, seed=1)))
    srv.drain()
    torch.cuda.synchronize(device)
    wl = serve.poisson_workload(n_requests, rate, shapes, branch, frac_continue=frac_continue, n_steps=500,
                                ds=50.0, seed=seed)
    st0 = dict(srv.stats)
    wall = serve.run_workload(srv, wl)
    srv.stop()
    reqs = [r for _, r in wl]
    con = [r for r in reqs if r.kind == "continue"]
    ok_con = [r for r in con if r.error is None and r.result["converged"] and r.result["residual"] <= 1e-10]
    ok_int = [r for r in reqs if r.kind == "integrate" and r.error is None and np.isfinite(r.result["X"]).all()]
    lat = serve.latency_report(reqs)
    return {"solves_per_s": (len(ok_con) + len(ok_int)) / wall, "requests": len(reqs), "wall_s": wall,
            "offered_rate_per_s": rate, "p50_ms": lat.get("p50_ms"), "p99_ms": lat.get("p99_ms"),
            "continuation": dict(serve.latency_report(con), n=len(con), converged_le_1e10=len(ok_con),
                                 max_residual=max((r.result["residual"] for r in con if r.result), default=None),
                                 mean_corrector_iters=float(np.mean([r.result["corrector_iters"] for r in con
                                                                     if r.result])) if con else None),
            "integration": dict(serve.latency_report([r for r in reqs if r.kind == "integrate"]),
                                n=len(reqs) - len(con), finite=len(ok_int)),
            "errors": sum(r.error is not None for r in reqs),
            "batching": {k: srv.stats[k] - st0[k] for k in srv.stats},
            "shapes": [f"{a}x{b}" for a, b in shapes], "branch_seconds": t_branch,
            "precision": {"integration": srv.int_precision + " (FP32 nonlinear term, FP64 implicit solves)",
                          "continuation": "FP32 nonlinear term inside the Jacobian products, FP64 residual <= 1e-10"},
            "chain_layout": srv.chain_layout, "tangent_rtol": srv.tangent_rtol, "con_workers": con_workers,
            "workload": "Poisson arrivals; 70% pseudo-arclength steps (ds=50, sign +-1) from steady states at "
                        "Ra_T=9000 on the Tau=1 branch, 30% 500-step integrations (dt=1e-3, Ra_T~U[8500,9500]) from "
                        "seeded states; N_r in {20,28,36,48}, N_theta in {64,128,256,512}; Ra_S=500, Pr=1, d=2"}


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

    # warm-up
    for _ in range(args.warmup):
        plan.step(Xa, Ra, Ras, nsteps=chunk, out=Xb)
        Xa, Xb = Xb, Xa
    torch.cuda.synchronize()

    # ---- timed region (device-resident): K bench steps, L2 flushed between them (outside the events) --
    clocks = ClockSampler(device.index or 0)
    clocks.start()
    barrier(ws)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        flush.zero_()
        evs[i][0].record(stream)
        plan.step(Xa, Ra, Ras, nsteps=chunk, out=Xb)
        evs[i][1].record(stream)
        Xa, Xb = Xb, Xa
    torch.cuda.synchronize()
    barrier(ws)
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
    roofline = {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved_gbs / hbm_peak, "traffic": traffic, "kernel": dom,
                "peak_source": hbm_src, "algorithmic_bytes_per_launch": kbytes,
                "launch_ms": kavg[dom],
                "fp64": {"achieved_gflops": kflops / dom_s / 1e9, "peak_gflops": fp64.value,
                         "frac": kflops / dom_s / 1e9 / fp64.value,
                         "peak_source": "measured live (sdd_measure_fp64_peak FMA loop)",
                         "algorithmic_flops_per_launch": kflops},
                "kernel_ms_per_step": kstep,
                "stage_ms_per_step": dict(zip(["nonlinear_term", "rhs", "implicit_solves"], ms3)),
                "step_fp64_gflops": step_flops / (ms_total * 1e-3 / (args.steps * chunk)) / 1e9}

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
        # space), FP32 nonlinear term, right-hand sides and h matvecs inside the Jacobian products (FP64
        # chains, Krylov basis and residual), FP64 residual <= 1e-10
        nb = 64
        planm = Plan(M, N_r, w["d"], 1.0, w["Pr"], w["Tau"], precision="mixed", device=device)
        planm.set_chain_layout(4)      # whole chains, split rows: measured best for the 64-shell Newton batch
        pert = torch.from_numpy(np.stack([seeded_state(M, N_r - 1, 500 + i) for i in range(nb)])).to(device)
        Xb0 = X_after.reshape(1, -1) + pert
        Rab = torch.linspace(7000.0, 9000.0, nb, dtype=torch.float64, device=device)
        planm.newton(Xb0.clone(), Rab, Ras, tol=1e-10, restart=50, max_newton=1, mixed_matvec=2)  # warm-up
        Xb = Xb0.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rb = planm.newton(Xb, Rab, Ras, tol=1e-10, restart=50, gmres_rtol=1e-4, max_newton=20, mixed_matvec=2)
        torch.cuda.synchronize()
        tb = time.perf_counter() - t0
        newton["batched"] = {"solves_per_s": nb / tb, "seconds": tb, "shells": nb, "mixed_matvec": 2,
                             "converged": sum(r["converged"] for r in rb),
                             "max_residual": max(r["residual"] for r in rb), "matvecs": rb[0]["matvecs"],
                             "vs_plain_single_shell": (nb / tb) / (1.0 / tn),
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
        bm = bench_batched(device, "mixed")
        bd = bench_batched(device, "fp64")
        plain = value / ws
        batched = {"mixed": bm, "fp64": bd,
                   "mixed_vs_plain_single_shell": bm["shell_steps_per_s"] / plain,
                   "fp64_vs_plain_single_shell": bd["shell_steps_per_s"] / plain,
                   "cpu_baseline": None if args.no_cpu else bench_batched_cpu(),
                   "workload": "64 shells, N_r in {20,24,30,36}, N_theta in {64,128,256,384}, Ra_T ~ U[6000,12000],"
                               " Ra_S=500, Pr=1, Tau=0.01, dt=1e-3, 1000 steps each (seed 1234)"}

    served = None
    if rank == 0 and not args.no_served:
        served = bench_served(device, n_requests=args.served_requests)

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
                "roofline": roofline, "cpu_baseline": cpu, "clocks": ck, "newton": newton, "mixed": mixed,
                "batched": batched,
                "served": served}
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def profile_newton_batch():
    """One Newton iteration (residual, one GMRES(50) solve, update) of the 64-shell batched Newton workload
    inside an NVTX range "newton_batched", for a kernel launch list of the batched Jacobian products:
    ncu --nvtx --nvtx-include "newton_batched/" ... python bench.py --profile-newton-batch.  The start: the
    seeded shell after 2000 IMEX steps of dt=5e-4 plus the 64 seeded perturbations of the bench workload."""
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
    q.newton(Xb0.clone(), Rab, Ras, tol=1e-10, restart=50, max_newton=1, mixed_matvec=2)   # warm-up
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("newton_batched")
    r = q.newton(Xb0.clone(), Rab, Ras, tol=1e-10, restart=50, max_newton=1, mixed_matvec=2)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    print(json.dumps({"profile": "newton_batched", "shells": nb, "jacobian_products": r[0]["matvecs"]}))
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
    ap.add_argument("--profile-newton-batch", action="store_true")
    args = ap.parse_args()
    if args.profile_newton_batch:
        return profile_newton_batch()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return bench_reference(args)
    return bench_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
