"""Many independent shells of uneven (N_r, N_theta) and Ra_T advanced together on one GPU.

The reference advances one shell per process (Main.py:228-329).  Here a batch of shells is grouped by
shape; every group shares one device plan (the operators depend on (N_fm, N_r, d, dt, Pr, Tau) only, not
on Ra_T, Main.py:179-225) and holds its shells' states contiguously on the device.  A batched step
launches the plan's kernels once per group; ``capture`` records ``steps_per_launch`` steps of every group
into ONE CUDA graph, each group on its own stream branch so the groups run concurrently, and ``replay``
then advances every shell with a single graph launch.  ``autotune`` picks each group's chain layout
(one lane per matrix row, or rows split over four warps) by timing the captured graph, and records the
choice.
"""
import time

import numpy as np

from .seeds import seeded_state

from .plan import Plan


def _torch():
    import torch
    return torch


class _Group:
    def __init__(self, plan, idx, X, Ra, Ra_s, device, priority=0):
        torch = _torch()
        self.plan = plan
        self.idx = list(idx)                 # positions of the shells in the caller's list
        self.X = torch.from_numpy(np.ascontiguousarray(np.stack(X))).to(device)
        self.Ra = torch.tensor(Ra, dtype=torch.float64, device=device)
        self.Ras = torch.tensor(Ra_s, dtype=torch.float64, device=device)
        self.stream = torch.cuda.Stream(device=device, priority=priority)
        self.priority = priority

    @property
    def shape(self):
        return (self.plan.N_r, self.plan.N_fm)


class ShellBatch:
    """shells: list of dicts with keys N_r, N_theta, Ra (Ra_T) and optionally Ra_s, X (initial state,
    flat numpy array in the reference layout; seeded if absent) and symmetric."""

    def __init__(self, shells, d=2.0, dt=1e-3, Pr=1.0, Tau=0.01, Ra_s=500.0, precision="mixed",
                 device=None, seed=1234, max_group=None, priorities=False, tuning=None):
        torch = _torch()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.d, self.dt, self.Pr, self.Tau, self.precision = d, dt, Pr, Tau, precision
        self.n_shells = len(shells)
        groups = {}
        rng = np.random.default_rng(seed)
        for i, s in enumerate(shells):
            key = (int(s["N_r"]), int(s["N_theta"]), bool(s.get("symmetric", False)))
            groups.setdefault(key, []).append(i)
        self.groups = []
        # every group has its own plan (its own workspace: groups run concurrently); groups larger than
        # max_group are split into sub-groups on separate streams
        parts = []
        for (N_r, M, sym), idx in sorted(groups.items(), key=lambda kv: -kv[0][1] * kv[0][0]):
            step = max_group if max_group else len(idx)
            parts += [((N_r, M, sym), idx[k:k + step]) for k in range(0, len(idx), step)]
        # optional stream priorities: the costliest groups (M nr^2 per shell x shells) on high-priority
        # streams, so the critical path of the graph is not delayed by the small groups
        cost = [M * (N_r - 1) ** 2 * len(idx) for (N_r, M, _), idx in parts]
        ranked = sorted(range(len(parts)), key=lambda k: -cost[k])
        high = set(ranked[:max(1, len(parts) // 4)]) if priorities else set()
        for k, ((N_r, M, sym), idx) in enumerate(parts):
            plan = Plan(M, N_r, d, dt, Pr, Tau, symmetric=sym, precision=precision, device=self.device)
            X = []
            for i in idx:
                x0 = shells[i].get("X")
                X.append(np.asarray(x0, dtype=np.float64) if x0 is not None else
                         _seeded(M, N_r - 1, rng))
            g = _Group(plan, idx, X, [float(shells[i]["Ra"]) for i in idx],
                       [float(shells[i].get("Ra_s", Ra_s)) for i in idx], self.device,
                       priority=-1 if k in high else 0)
            plan.reserve(len(idx))
            self.groups.append(g)
        # Starting point of the tuning (measured on the 64-shell mixed batch of N_r in {20..36}, N_theta in
        # {64..384}): the groups' launches share the GPU inside one graph, so the nonlinear term runs as the
        # fused row kernel once the batch fills the SMs; the chains run in the reference's order of
        # operations, a shell's three chains of one parity per CTA (layout 8: 4 nr^2 multiply-adds per mode
        # instead of 7; the library runs layout 5 where the right-hand side is fused or FP32, and layout 6
        # where the three rings do not fit a CTA), and chunked chains for N_theta >= 256 with the FP32
        # nonlinear term, where the long chains of the largest shells set the critical path, each chunk in
        # the reference's order too (layout 10: 96.0k shell-steps/s with it on every group against 88.3k
        # for the pre-pass chunks of layout 2); in FP64 the nonlinear term dominates and chunking does not
        # pay.
        sms = _torch().cuda.get_device_properties(self.device).multi_processor_count
        total_rows = sum(g.plan.nr * len(g.idx) for g in self.groups)
        for g in self.groups:
            g.plan.set_chain_layout(10 if (precision == "mixed" and g.plan.N_fm >= 256) else 8)
            g.plan.set_fx_split(1 if 2 * total_rows > sms else 0)
        self.graph = None
        self.steps_per_launch = 0
        self.tuning = {}
        if tuning:
            self.apply_tuning(tuning)

    def apply_tuning(self, tuning):
        """Per-shape kernel choices of an earlier autotune() (its returned dict), e.g. of a scratch batch
        of the same shapes.  A batch timed straight after its own tuning ran some 8% slower than a fresh
        batch with the same choices; timed again later it ran at the fresh batch's speed (6.65 vs 6.66 ms a
        launch), so the difference was the GPU's clock state after the tuning bursts, not the batch."""
        for g in self.groups:
            c = tuning.get("N_r=%d,N_theta=%d" % g.shape)
            if c:
                g.plan.set_chain_layout(int(c["chain_layout"]))
                g.plan.set_fx_split(int(c["fx_split"]))
                for cset, kc in enumerate(c.get("chunk_length", (0, 0))):
                    if g.plan.chunk_length[cset] != int(kc):
                        g.plan.set_chunk_length(cset, int(kc))
                self.tuning["N_r=%d,N_theta=%d" % g.shape] = dict(c)
        self.graph = None

    # ---- eager ---------------------------------------------------------------------------------
    def step(self, nsteps=1):
        """Advance every shell by nsteps (one launch sequence per group, groups on their own streams)."""
        torch = _torch()
        main = torch.cuda.current_stream(self.device)
        for g in self.groups:
            g.stream.wait_stream(main)
            with torch.cuda.stream(g.stream):
                g.plan.step(g.X, g.Ra, g.Ras, nsteps=nsteps, out=g.X)
        for g in self.groups:
            main.wait_stream(g.stream)

    # ---- graph ---------------------------------------------------------------------------------
    def capture(self, steps_per_launch=10):
        """Record steps_per_launch steps of every group into one CUDA graph (groups as parallel branches)."""
        torch = _torch()
        saved = [g.X.clone() for g in self.groups]
        self.step(1)                      # kernel attributes and workspaces are set up outside capture
        for g, x in zip(self.groups, saved):
            g.X.copy_(x)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        cap = torch.cuda.Stream(device=self.device)
        with torch.cuda.stream(cap):
            with torch.cuda.graph(g, stream=cap, capture_error_mode="thread_local"):
                for grp in self.groups:
                    grp.stream.wait_stream(cap)
                    with torch.cuda.stream(grp.stream):
                        grp.plan.step(grp.X, grp.Ra, grp.Ras, nsteps=steps_per_launch, out=grp.X)
                for grp in self.groups:
                    cap.wait_stream(grp.stream)
        self.graph = g
        self.steps_per_launch = steps_per_launch
        return g

    def replay(self, launches=1):
        for _ in range(launches):
            self.graph.replay()

    # ---- tuning --------------------------------------------------------------------------------
    def _time_graph(self, reps):
        """Seconds per launch of the current choices: best of two event-timed runs of `reps` launches."""
        torch = _torch()
        self.capture(self.steps_per_launch or 5)
        self.graph.replay()
        torch.cuda.synchronize(self.device)
        stream = torch.cuda.current_stream(self.device)
        best = float("inf")
        for _ in range(2):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                self.graph.replay()
            e1.record(stream)
            torch.cuda.synchronize(self.device)
            best = min(best, e0.elapsed_time(e1) * 1e-3 / reps)
        return best

    def autotune(self, steps_per_launch=5, reps=3, layouts=(1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11), fx_modes=(1, 2),
                 chunk_scales=(0.6, 1.6), min_gain=0.015):
        """Greedy per-group choice of the chain layout, then of the nonlinear-term kernel (fused or split),
        then, for a group whose chains run chunked, of the chunk length (the rule's times chunk_scales),
        minimising the time of one graph launch; a change is kept only if it gains more than min_gain (the
        groups share the GPU, so single timings are noisy), and the starting choices are kept when the
        tuned ones do not beat them on a final re-measurement.  The shells' states are restored
        afterwards: tuning does not advance them."""
        saved = [g.X.clone() for g in self.groups]
        self.steps_per_launch = steps_per_launch
        start = [(g.plan.chain_layout, g.plan.fx_split, list(g.plan.chunk_length)) for g in self.groups]
        t_start = best = self._time_graph(reps)
        for g in self.groups:
            choice = g.plan.chain_layout
            for lay in layouts:
                if lay == choice:
                    continue
                g.plan.set_chain_layout(lay)
                t = self._time_graph(reps)
                if t < best * (1.0 - min_gain):
                    best, choice = t, lay
            g.plan.set_chain_layout(choice)
            fx_choice = g.plan.fx_split
            for fx in fx_modes:
                if fx == fx_choice:
                    continue
                g.plan.set_fx_split(fx)
                t = self._time_graph(reps)
                if t < best * (1.0 - min_gain):
                    best, fx_choice = t, fx
            g.plan.set_fx_split(fx_choice)
            lay, kc0, _ = g.plan.chain_choice(len(g.idx))
            if lay in (2, 3, 10, 11) and chunk_scales:
                cset = 1 if lay in (3, 11) else 0
                kc_choice = g.plan.chunk_length[cset]
                for sc in chunk_scales:
                    kc = max(2, int(round(kc0 * sc)))
                    if kc == kc0:
                        continue
                    try:
                        g.plan.set_chunk_length(cset, kc)
                    except Exception:            # noqa: BLE001 - outside the allowed chunk counts
                        continue
                    t = self._time_graph(reps)
                    if t < best * (1.0 - min_gain):
                        best, kc_choice = t, kc
                g.plan.set_chunk_length(cset, kc_choice)
        t_tuned = self._time_graph(reps)
        if t_tuned > t_start:
            for g, (lay, fx, kcs) in zip(self.groups, start):
                g.plan.set_chain_layout(lay)
                g.plan.set_fx_split(fx)
                for cset, kc in enumerate(kcs):
                    if g.plan.chunk_length[cset] != kc:
                        g.plan.set_chunk_length(cset, kc)
        for g in self.groups:
            self.tuning["N_r=%d,N_theta=%d" % g.shape] = {"chain_layout": g.plan.chain_layout,
                                                          "fx_split": g.plan.fx_split,
                                                          "chunk_length": list(g.plan.chunk_length)}
        for g, x in zip(self.groups, saved):
            g.X.copy_(x)
        self.capture(steps_per_launch)
        return dict(self.tuning, seconds_per_launch=min(t_start, t_tuned), seconds_per_launch_start=t_start)

    # ---- results -------------------------------------------------------------------------------
    def states(self):
        """Per-shell states (numpy), in the caller's order."""
        out = [None] * self.n_shells
        for g in self.groups:
            Xh = g.X.cpu().numpy()
            for k, i in enumerate(g.idx):
                out[i] = Xh[k].copy()
        return out


def _seeded(M, nr, rng):
    return seeded_state(M, nr, rng)


def config4_shells(n=64, seed=1234):
    """The batched workload: N_r in {20,24,30,36}, N_theta in {64,128,256,384}, Ra_T ~ U[6000,12000]."""
    rng = np.random.default_rng(seed)
    Nr = rng.choice([20, 24, 30, 36], size=n)
    Nt = rng.choice([64, 128, 256, 384], size=n)
    Ra = rng.uniform(6000.0, 12000.0, size=n)
    return [dict(N_r=int(a), N_theta=int(b), Ra=float(c)) for a, b, c in zip(Nr, Nt, Ra)]
