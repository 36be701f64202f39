"""Continuous-batching request server for time integrations and pseudo-arclength continuation steps.

The reference runs one shell per process and one request at a time (Main.py:228, 742, 958).  Here one
process drives one GPU:

* An integration request (N_r, N_theta, Ra_T, initial state, n_steps) joins the device-resident batch of
  its shape at the next quantum boundary and leaves it when its steps are done (continuous batching): every
  quantum advances all active shells of a shape with one batched launch sequence (``Plan.step``).
* A continuation request (a steady state on a branch, Ra_T, sign, ds) is one ``_ContinC`` step
  (Main.py:742-955) on the GPU (``Plan.contin_step``); waiting requests of one shape are batched into one
  call (each shell keeps its own Krylov space and control flow).
* The two kinds run on host threads with their own CUDA streams (one integration worker, ``con_workers``
  continuation workers that never take the same shape at once), so their work overlaps on the device
  (the C calls release the GIL).
* Admission is FIFO against a device-memory budget: a request is admitted when the bytes it needs (its
  state and its share of the workspaces, plus the operators of a shape seen for the first time) fit.
* Results do not depend on the mix: no arithmetic crosses shells, every reduction has a fixed order, and
  the plans' chain layout is fixed (the automatic choice would depend on the batch size).

Latency of a request = completion time - submission time; the server records admission, start (first
device work) and completion times, so a latency splits into queue time (submission to start) and device
time (start to completion) for p50/p99 reporting.

Failure paths (the reference's own exits are Main.py:541-544, 888-899, 923): a request whose state is or
becomes non-finite completes with an error instead of a result; a continuation step whose corrector does
not converge completes with an error; ``cancel`` retires a queued request at once and an in-flight one at
its next quantum boundary (integrations) or when its batched call returns (continuations).
"""
import collections
import itertools
import threading
import time

import numpy as np

from .plan import Plan
from .seeds import seeded_state


def _torch():
    import torch
    return torch


class Request:
    """kind "integrate": n_steps IMEX steps from X (seeded if None).  kind "continue": one arclength step
    from the steady state X at Ra with (sign, ds).  After completion ``result`` holds X, Ra and details."""
    _ids = itertools.count()

    def __init__(self, kind, N_r, N_theta, Ra, X=None, n_steps=500, sign=1.0, ds=50.0, seed=None):
        if kind not in ("integrate", "continue"):
            raise ValueError(kind)
        self.id = next(Request._ids)
        self.kind, self.N_r, self.N_theta, self.Ra = kind, int(N_r), int(N_theta), float(Ra)
        self.X, self.n_steps, self.sign, self.ds, self.seed = X, int(n_steps), float(sign), float(ds), seed
        self.t_submit = self.t_admit = self.t_start = self.t_done = None
        self.result = None
        self.error = None
        self.cancelled = False
        self._bytes = 0
        self.done = threading.Event()

    @property
    def shape(self):
        return (self.N_r, self.N_theta)

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_submit

    @property
    def queue_time(self):
        """Submission to the start of the request's first device work."""
        return None if self.t_start is None else self.t_start - self.t_submit

    @property
    def device_time(self):
        """Start of the request's first device work to completion."""
        return None if self.t_start is None or self.t_done is None else self.t_done - self.t_start


def _seeded(M, nr, seed):
    return seeded_state(M, nr, seed)


class _IntGroup:
    """Device-resident batch of the active integration requests of one shape (compact slots)."""

    def __init__(self, plan, device):
        torch = _torch()
        self.plan, self.device = plan, device
        self.cap = 0
        self.X = torch.empty((0, plan.n_state), dtype=torch.float64, device=device)
        self.Ra = torch.empty(0, dtype=torch.float64, device=device)
        self.Ras = torch.empty(0, dtype=torch.float64, device=device)
        self.reqs = []
        self.left = []

    def add(self, req, X0, Ra_s):
        torch = _torch()
        n = len(self.reqs)
        if n == self.cap:
            cap = max(4, 2 * self.cap)
            X = torch.empty((cap, self.plan.n_state), dtype=torch.float64, device=self.device)
            Ra = torch.empty(cap, dtype=torch.float64, device=self.device)
            Ras = torch.empty(cap, dtype=torch.float64, device=self.device)
            if n:
                X[:n].copy_(self.X[:n])
                Ra[:n].copy_(self.Ra[:n])
                Ras[:n].copy_(self.Ras[:n])
            self.X, self.Ra, self.Ras, self.cap = X, Ra, Ras, cap
            self.plan.reserve(cap)
        self.X[n].copy_(torch.from_numpy(np.ascontiguousarray(X0, dtype=np.float64)))
        self.Ra[n] = req.Ra
        self.Ras[n] = Ra_s
        self.reqs.append(req)
        self.left.append(req.n_steps)

    def remove(self, i):
        """swap-remove slot i (keeps the active slots contiguous)"""
        last = len(self.reqs) - 1
        if i != last:
            self.X[i].copy_(self.X[last])
            self.Ra[i] = self.Ra[last]
            self.Ras[i] = self.Ras[last]
            self.reqs[i], self.left[i] = self.reqs[last], self.left[last]
        self.reqs.pop()
        self.left.pop()


class Server:
    """Request server over one GPU.  Integrations use plans with step dt and nonlinear-term precision
    ``int_precision``; continuation steps use plans with dt = 1 (Main.py:430, PFX over one unit of time),
    an FP64 residual <= tol, and inside the Jacobian products the FP32 nonlinear term when ``con_mixed`` is
    1 (or True), FP32 right-hand sides and h = Linv g matvecs as well when it is 2 (the default), and an FP32
    Krylov basis too when it is 3 (a few ms lower p50 in the served mix, but one corrector in about 20k
    served steps ended on a non-finite state with it, none with 2).
    Integrations default to the mixed form (FP32 nonlinear term, FP64 implicit solves: 1.7x the served
    integration throughput of FP64 at these sizes; its trajectory error against FP64 is checked by the
    mixed-precision tests).  Every plan has the fixed chain layout ``chain_layout`` (default: chunked, the
    lowest latency at the served batch sizes); the tangent of each arclength step is solved to
    ``tangent_rtol`` (it only seeds the predictor: the corrector still converges to tol)."""

    def __init__(self, d=2.0, Pr=1.0, Tau=1.0, Ra_s=500.0, dt=1e-3, int_precision="mixed", con_mixed=2,
                 memory_budget=None, quantum=50, max_batch=16, device=None, chain_layout=2, tol=1e-10,
                 restart=50, con_workers=4, tangent_rtol=1e-4):
        torch = _torch()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.d, self.Pr, self.Tau, self.Ra_s, self.dt = d, Pr, Tau, Ra_s, dt
        self.int_precision, self.con_mixed = int_precision, int(con_mixed)
        if self.con_mixed not in (0, 1, 2, 3):
            raise ValueError("con_mixed: expected False/True, 0, 1, 2 or 3")
        self.quantum, self.max_batch, self.con_workers = int(quantum), int(max_batch), int(con_workers)
        self.chain_layout, self.tol, self.restart, self.tangent_rtol = chain_layout, tol, restart, tangent_rtol
        if memory_budget is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            memory_budget = int(0.5 * free)
        self.budget = int(memory_budget)
        self.used = 0              # bytes held by admitted requests
        self._active = 0           # admitted requests not yet finished
        self.resident = 0          # bytes of the plans' operators (kept for the server's lifetime)
        self._plans = {}
        self._shapes = set()       # (kind, shape) whose operators are counted in resident
        self._plan_lock = threading.Lock()
        self._cv = threading.Condition()
        self._pending = {"integrate": collections.deque(), "continue": collections.deque()}
        self._groups = {}
        self._waiting = collections.OrderedDict()
        self._con_inflight = set()   # shapes a continuation worker is solving (one worker per plan)
        self._int_joining = {}       # integration requests admitted, waiting for their group's boundary
        self.worker_error = None
        self._running = False
        self._threads = []
        self.completed = []
        self.stats = {"int_quanta": 0, "int_steps": 0, "con_calls": 0, "con_shells": 0, "rejected": 0}

    # ---- plans and memory ----------------------------------------------------------------------------
    def _plan(self, kind, N_r, M):
        """The server's own plan for (kind, shape): private to the server, so its fixed chain layout does
        not change plans used elsewhere, and the two worker threads never share a plan."""
        key = (kind, N_r, M)
        with self._plan_lock:
            p = self._plans.get(key)
            if p is None:
                if kind == "integrate":
                    p = Plan(M, N_r, self.d, self.dt, self.Pr, self.Tau, precision=self.int_precision,
                             device=self.device)
                else:
                    p = Plan(M, N_r, self.d, 1.0, self.Pr, self.Tau,
                             precision="mixed" if self.con_mixed else "fp64", device=self.device)
                if self.chain_layout is not None:
                    p.set_chain_layout(self.chain_layout)
                self._plans[key] = p
            return p

    def request_bytes(self, req):
        """Device bytes a request holds while admitted: its state and its share of the step workspace
        (FX outputs, right-hand sides, chain pre-pass), plus for continuation the Krylov basis (restart+1
        vectors of n+1), the bordered-system vectors and the base-state caches."""
        M, nr = req.N_theta, req.N_r - 1
        n = 3 * M * nr
        per = 8 * (8 * n + 9 * nr * (3 * M // 2 + 1))
        if req.kind == "continue":
            per += 8 * ((self.restart + 12) * (n + 1) + 2 * 9 * nr * (3 * M // 2 + 1))
        return per

    @staticmethod
    def plan_bytes(req):
        """Device bytes of a plan's operators (dense radial inverses and fused chain tables per mode)."""
        M, nr = req.N_theta, req.N_r - 1
        return 8 * (7 * M * nr * nr + 16 * nr * nr)

    def _try_admit(self, req):
        """True when admitted, False to wait for memory, "reject" when the request can never fit (the
        operators of admitted shapes stay resident, so that bound only grows)."""
        key = (req.kind, req.shape)
        stat = 0 if key in self._shapes else self.plan_bytes(req)
        need = self.request_bytes(req)
        if self.resident + stat + need > self.budget:
            return "reject"
        if self.resident + stat + self.used + need > self.budget:
            return False
        self._shapes.add(key)
        self.resident += stat
        self.used += need
        self._active += 1
        req._bytes = need
        req.t_admit = time.perf_counter()
        return True

    def _release(self, req):
        """Returns an admitted request's bytes to the budget (used by tests of the admission logic)."""
        with self._cv:
            self.used -= req._bytes
            req._bytes = 0
            self._cv.notify_all()

    # ---- API -----------------------------------------------------------------------------------------
    def submit(self, req):
        req.t_submit = time.perf_counter()
        with self._cv:
            self._pending[req.kind].append(req)
            self._cv.notify_all()
        return req

    def cancel(self, req):
        """Retires a request: a queued one (not yet admitted, or admitted and waiting for its batch) at once,
        an integration in flight at its group's next quantum boundary, a continuation in flight when its
        batched call returns.  The request completes with error "cancelled".  Returns True if it was still
        pending or in flight."""
        with self._cv:
            if req.done.is_set():
                return False
            req.cancelled = True
            q = self._pending[req.kind]
            if req in q:                                  # never admitted: no bytes to return
                q.remove(req)
                req.error = "cancelled"
                req.t_done = time.perf_counter()
                req.done.set()
                self._cv.notify_all()
                return True
            lst = (self._waiting if req.kind == "continue" else self._int_joining).get(req.shape, [])
            waiting = req in lst
            if waiting:
                lst.remove(req)
        if waiting:
            self._finish(req, error="cancelled")
        return True

    def start(self):
        self._running = True
        for fn in [self._int_loop] + [self._con_loop] * self.con_workers:
            t = threading.Thread(target=fn, daemon=True)
            t.start()
            self._threads.append(t)
        return self

    def stop(self):
        with self._cv:
            self._running = False
            self._cv.notify_all()
        for t in self._threads:
            t.join()
        self._threads = []

    def drain(self, timeout=None):
        """Wait until every submitted request has completed (or been rejected)."""
        t0 = time.perf_counter()
        with self._cv:
            while (any(self._pending.values()) or self._active) and self.worker_error is None:
                left = None if timeout is None else timeout - (time.perf_counter() - t0)
                if left is not None and left <= 0:
                    return False
                self._cv.wait(timeout=0.05 if left is None else min(0.05, left))
        return self.worker_error is None

    def _worker_failed(self, kind, exc):
        """A worker thread hit an unexpected error: every request it holds or would take fails with it, and
        ``worker_error`` records it (drain() returns instead of waiting)."""
        msg = "%s worker failed: %r" % (kind, exc)
        self.worker_error = msg
        owned = []
        with self._cv:
            owned += list(self._pending[kind])
            self._pending[kind].clear()
            if kind == "integrate":
                for g in self._groups.values():
                    owned += list(g.reqs)
                    g.reqs, g.left = [], []
                for lst in self._int_joining.values():
                    owned += list(lst)
                self._int_joining.clear()
            else:
                for lst in self._waiting.values():
                    owned += list(lst)
                self._waiting.clear()
        for req in owned:
            if req.t_admit is None:                     # never admitted: no bytes to return
                req.error = msg
                req.t_done = time.perf_counter()
                req.done.set()
            else:
                self._finish(req, error=msg)

    def _finish(self, req, result=None, error=None):
        req.result, req.error = result, error
        req.t_done = time.perf_counter()
        with self._cv:
            self.used -= req._bytes
            req._bytes = 0
            self._active -= 1
            self.completed.append(req)
            self._cv.notify_all()
        req.done.set()

    def _admit_kind(self, kind):
        """Moves admissible pending requests of one kind (FIFO, head of line blocks) out of the queue."""
        out = []
        q = self._pending[kind]
        while q:
            r = self._try_admit(q[0])
            if r == "reject":
                req = q.popleft()
                self.stats["rejected"] += 1
                req.error = "request exceeds the device-memory budget"
                req.t_done = time.perf_counter()
                req.done.set()
                continue
            if not r:
                break
            out.append(q.popleft())
        return out

    # ---- integration worker --------------------------------------------------------------------------
    def _int_loop(self):
        """Continuous batching of integrations.  Every shape group runs on its own stream and advances
        independently: when a group's quantum (up to ``quantum`` steps of all its shells) has finished, its
        completed requests are retired, the requests admitted for its shape since then join, and the next
        quantum is launched.  Groups of different shapes overlap on the device and never wait for each
        other."""
        try:
            self._int_loop_body()
        except Exception as e:                          # noqa: BLE001 - a dead worker fails its requests
            self._worker_failed("integrate", e)

    def _int_loop_body(self):
        torch = _torch()
        torch.cuda.set_device(self.device)
        streams, events, busy = {}, {}, {}
        joining = self._int_joining
        while True:
            with self._cv:
                new = self._admit_kind("integrate")
                idle = not new and not any(busy.values()) and not any(joining.values()) and \
                    not any(g.reqs for g in self._groups.values())
                if idle:
                    if not self._running and not self._pending["integrate"]:
                        return
                    self._cv.wait(timeout=0.01)
                    continue
            with self._cv:
                for req in new:
                    joining.setdefault(req.shape, []).append(req)
            progressed = False
            for shape in list(set(self._groups) | set(joining)):
                g = self._groups.get(shape)
                if busy.get(shape):
                    if not events[shape].query():
                        continue
                    busy[shape] = False
                    progressed = True
                    with torch.cuda.stream(streams[shape]):
                        i = 0
                        while i < len(g.reqs):
                            req = g.reqs[i]
                            if req.cancelled:
                                g.remove(i)
                                self._finish(req, error="cancelled")
                            elif g.left[i] <= 0:
                                X = g.X[i].cpu().numpy().copy()
                                g.remove(i)
                                if np.isfinite(X).all():
                                    self._finish(req, result={"X": X, "Ra": req.Ra, "steps": req.n_steps})
                                else:
                                    self._finish(req, error="non-finite state after %d steps" % req.n_steps)
                            else:
                                i += 1
                with self._cv:
                    joined = joining.pop(shape, [])
                for req in joined:
                    if req.cancelled:
                        self._finish(req, error="cancelled")
                        continue
                    try:
                        if g is None:
                            g = _IntGroup(self._plan("integrate", req.N_r, req.N_theta), self.device)
                            self._groups[shape] = g
                            streams[shape] = torch.cuda.Stream(device=self.device)
                            events[shape] = torch.cuda.Event()
                        X0 = req.X if req.X is not None else _seeded(req.N_theta, req.N_r - 1,
                                                                     req.seed if req.seed is not None else req.id)
                        with torch.cuda.stream(streams[shape]):
                            g.add(req, X0, self.Ra_s)
                    except Exception as e:          # noqa: BLE001 - report per request
                        self._finish(req, error=repr(e))
                if g is None or not g.reqs:
                    continue
                na = len(g.reqs)
                q = min(self.quantum, min(g.left))
                now = time.perf_counter()
                for req in g.reqs:
                    if req.t_start is None:
                        req.t_start = now
                try:
                    with torch.cuda.stream(streams[shape]):
                        g.plan.step(g.X[:na], g.Ra[:na], g.Ras[:na], nsteps=q, out=g.X[:na])
                        events[shape].record(streams[shape])
                except Exception as e:          # noqa: BLE001 - fail the group's requests, keep serving
                    while g.reqs:
                        req = g.reqs[-1]
                        g.remove(len(g.reqs) - 1)
                        self._finish(req, error=repr(e))
                    continue
                busy[shape] = True
                progressed = True
                self.stats["int_quanta"] += 1
                self.stats["int_steps"] += q * na
                g.left = [x - q for x in g.left]
            if not progressed:
                time.sleep(0.0002)

    # ---- continuation worker -------------------------------------------------------------------------
    def _con_loop(self):
        try:
            self._con_loop_body()
        except Exception as e:                          # noqa: BLE001 - a dead worker fails its requests
            self._worker_failed("continue", e)

    def _con_loop_body(self):
        torch = _torch()
        torch.cuda.set_device(self.device)
        stream = torch.cuda.Stream(device=self.device)
        with torch.cuda.stream(stream):
            while True:
                with self._cv:
                    for req in self._admit_kind("continue"):
                        self._waiting.setdefault(req.shape, []).append(req)
                    shape = None
                    oldest = None
                    for sh, lst in self._waiting.items():     # oldest waiting shape no other worker holds
                        if lst and sh not in self._con_inflight and (oldest is None or lst[0].t_submit < oldest):
                            shape, oldest = sh, lst[0].t_submit
                    if shape is None:
                        if not self._running and not self._pending["continue"] and not any(self._waiting.values()):
                            return
                        self._cv.wait(timeout=0.01)
                        continue
                    batch = self._waiting[shape][:self.max_batch]
                    del self._waiting[shape][:len(batch)]
                    self._con_inflight.add(shape)
                t0 = time.perf_counter()
                for req in batch:
                    req.t_start = t0
                try:
                    plan = self._plan("continue", *shape)
                    X = torch.from_numpy(np.stack([np.asarray(r.X, dtype=np.float64) for r in batch])).to(self.device)
                    Ra = torch.tensor([r.Ra for r in batch], dtype=torch.float64, device=self.device)
                    Xd, res = plan.contin_step(X, Ra, self.Ra_s, [r.sign for r in batch], [r.ds for r in batch],
                                               tol=self.tol, restart=self.restart, mixed_matvec=self.con_mixed,
                                               tangent_rtol=self.tangent_rtol)
                    Xh, Rah, Xdh = X.cpu().numpy(), Ra.cpu().numpy(), Xd.cpu().numpy()
                    with self._cv:
                        self.stats["con_calls"] += 1
                        self.stats["con_shells"] += len(batch)
                    for k, req in enumerate(batch):
                        if req.cancelled:
                            self._finish(req, error="cancelled")
                        elif not (np.isfinite(Xh[k]).all() and np.isfinite(Rah[k])):
                            self._finish(req, error="non-finite state")
                        elif not res[k]["converged"]:
                            self._finish(req, error="corrector did not converge (|F| = %.3e after %d halvings)"
                                         % (res[k]["residual"], res[k]["halvings"]))
                        else:
                            self._finish(req, result={"X": Xh[k].copy(), "Ra": float(Rah[k]),
                                                      "X_dot": Xdh[k].copy(), **res[k]})
                except Exception as e:              # noqa: BLE001 - report per request
                    for req in batch:
                        self._finish(req, error=repr(e))
                finally:
                    with self._cv:
                        self._con_inflight.discard(shape)
                        self._cv.notify_all()


# ---- workload helpers ---------------------------------------------------------------------------------
def branch_states(shapes, Ra=9000.0, d=2.0, Pr=1.0, Tau=1.0, Ra_s=500.0, device=None, source=None,
                  small=(16, 16), dt=5e-3, steps=40000, tol=1e-10, max_newton=30):
    """Steady convective states on one branch for every (N_r, N_theta) in shapes.

    The seed is ``source = (X, N_r, N_theta)`` (a steady state at Ra) or, when None, a shell of shape
    ``small`` time-stepped from a seeded state to saturation and polished by Newton.  Shapes are then
    taken in increasing size: each is interpolated (INTERP_RADIAL / INTERP_THETAS, Main.py:414-416) from the
    last converged one and polished by Newton-GMRES to an FP64 residual <= tol.
    Returns {shape: (X, residual)}; a shape whose Newton solve did not converge is left out."""
    torch = _torch()
    from . import Matrix_Operators as MO
    if source is None:
        N_r0, M0 = small
        p = Plan(M0, N_r0, d, dt, Pr, Tau, device=device)
        X = torch.from_numpy(_seeded(M0, N_r0 - 1, 31)).to(p.device).reshape(1, -1)
        X = p.step(X, Ra, Ra_s, nsteps=steps)
        p1 = Plan(M0, N_r0, d, 1.0, Pr, Tau, device=device)
        p1.newton(X, Ra, Ra_s, tol=tol, max_newton=max_newton)
        source = (X.cpu().numpy().ravel(), N_r0, M0)
    X0, N_r0, M0 = np.asarray(source[0], dtype=np.float64).ravel(), int(source[1]), int(source[2])
    out = {}
    for (N_r, M) in sorted(set((int(a), int(b)) for a, b in shapes), key=lambda s: (s[0] * s[1], s)):
        Xi = MO.INTERP_RADIAL(N_r, N_r0, X0, d) if N_r != N_r0 else X0.copy()
        Xi = MO.INTERP_THETAS(M, M0, Xi) if M != M0 else Xi
        pn = Plan(M, N_r, d, 1.0, Pr, Tau, device=device)
        Xt = torch.from_numpy(np.ascontiguousarray(Xi, dtype=np.float64)).to(pn.device).reshape(1, -1)
        r = pn.newton(Xt, Ra, Ra_s, tol=tol, max_newton=max_newton)[0]
        pn.close()
        if r["converged"]:
            X0, N_r0, M0 = Xt.cpu().numpy().ravel(), N_r, M
            out[(N_r, M)] = (X0.copy(), r["residual"])
    return out


def poisson_workload(n, rate, shapes, branch, frac_continue=0.7, n_steps=500, ds=50.0, seed=1234,
                     Ra_int=(8500.0, 9500.0)):
    """n requests with exponential inter-arrival times (mean 1/rate): a fraction frac_continue are
    arclength steps from the branch states (sign +-1, ds), the rest n_steps integrations from seeded states
    at Ra ~ U(Ra_int).  Returns [(arrival_offset_s, Request)]."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        shape = shapes[rng.integers(len(shapes))]
        if rng.random() < frac_continue:
            X, _ = branch[shape]
            req = Request("continue", shape[0], shape[1], 9000.0, X=X, sign=float(rng.choice([-1.0, 1.0])), ds=ds)
        else:
            req = Request("integrate", shape[0], shape[1], float(rng.uniform(*Ra_int)), n_steps=n_steps,
                          seed=int(rng.integers(1 << 30)))
        out.append((t, req))
    return out


def run_workload(server, workload):
    """Submits the requests at their arrival offsets (wall clock) and waits for all of them."""
    t0 = time.perf_counter()
    for off, req in workload:
        now = time.perf_counter() - t0
        if off > now:
            time.sleep(off - now)
        server.submit(req)
    server.drain()
    return time.perf_counter() - t0


def latency_report(reqs):
    """p50/p99/mean/max of the latency of the completed requests, and of its two parts: queue time
    (submission to first device work) and device time (first device work to completion)."""
    ok = [r for r in reqs if r.latency is not None and r.error is None]
    lat = np.array([r.latency for r in ok])
    if lat.size == 0:
        return {}
    out = {"n": int(lat.size), "p50_ms": float(np.percentile(lat, 50) * 1e3),
           "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
           "max_ms": float(lat.max() * 1e3)}
    for name in ("queue", "device"):
        v = np.array([getattr(r, name + "_time") for r in ok if getattr(r, name + "_time") is not None])
        if v.size:
            out[name + "_p50_ms"] = float(np.percentile(v, 50) * 1e3)
            out[name + "_p99_ms"] = float(np.percentile(v, 99) * 1e3)
    return out
