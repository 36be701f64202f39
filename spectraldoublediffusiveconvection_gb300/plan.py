"""Plans: device-resident operators for one (N_fm, N_r, d, dt, Pr, Tau, symmetric, precision).

A plan replaces the operator tuple of ``Build_Matrix_Operators`` (Main.py:179-225) on the GPU.  The
operators do not depend on Ra_T (it enters only through the buoyancy coupling, Main.py:271), so shells
that share (N_fm, N_r, d, dt, Pr, Tau) share one plan and are advanced as a batch.

All compute goes through libsdd_gb300 (C ABI, ``include/sdd_gb300.h``); torch provides device memory
and the current stream.
"""
import ctypes
import threading

import numpy as np

from . import _lib
from .operators import plan_arrays

_PREC = {"fp64": _lib.SDD_PREC_FP64, "mixed": _lib.SDD_PREC_MIXED}


def _torch():
    import torch
    return torch


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _stream(device):
    torch = _torch()
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


class Plan:
    """Device operators + workspace for shells of one shape and step.

    Parameters mirror ``Build_Matrix_Operators(N_fm, N_r, d, dt, Pr, Tau)`` plus ``symmetric`` and the
    nonlinear-term precision ("fp64" plain, "mixed" = FP32 nonlinear term / FP64 solves).
    """

    def __init__(self, N_fm, N_r, d, dt, Pr, Tau, symmetric=False, precision="fp64", device=None,
                 arrays=None):
        torch = _torch()
        if not torch.cuda.is_available():
            raise RuntimeError("a CUDA device is required (libsdd_gb300 has no CPU path)")
        if N_fm % 2 != 0:
            raise ValueError('The number of Fourier modes is not even %d' % N_fm)
        self.N_fm, self.N_r, self.d, self.dt, self.Pr, self.Tau = int(N_fm), int(N_r), float(d), float(dt), \
            float(Pr), float(Tau)
        self.nr = self.N_r - 1
        self.symmetric = bool(symmetric)
        self.precision = precision
        self.chain_layout = 0          # automatic (sdd_plan_set_chain_layout)
        self.chunk_length = [0, 0]     # steps per chunk of the two chunk sets, 0: the rule
        self.fx_split = 0              # automatic (sdd_plan_set_fx_split)
        self.tensor_cores = precision == "mixed"   # sdd_plan_set_tensor_cores
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.arrays = arrays if arrays is not None else plan_arrays(N_fm, N_r, d, dt, Pr, Tau)
        A = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in self.arrays.items()
             if isinstance(v, np.ndarray)}
        self._host = A
        desc = _lib.PlanDesc()
        desc.N_fm, desc.nr, desc.symmetric = self.N_fm, self.nr, int(self.symmetric)
        desc.precision = _PREC[precision]
        desc.dt, desc.Pr, desc.Tau = self.dt, self.Pr, self.Tau
        for name in ("Dr", "D2_r2", "ir4_r2", "D2_sine", "ir2_sine", "D2_A4", "ir2_A4", "ir4_A4", "rsq",
                     "dT0", "gr", "Linv_A4", "Linv_T", "Linv_S"):
            setattr(desc, name, _ptr(A[name]))
        if "nu_w" in A and "r_int" in A and "R" in A:      # diagnostics tables (optional)
            desc.nu_w, desc.r_int = _ptr(A["nu_w"]), _ptr(A["r_int"])
            desc.r_i, desc.r_o = float(A["R"][0]), float(A["R"][-1])
        h = ctypes.c_void_p()
        L = _lib.lib()
        with torch.cuda.device(self.device):
            _lib.check(L.sdd_plan_create(ctypes.byref(desc), ctypes.byref(h)), "sdd_plan_create")
        self._h = h
        self._L = L
        self.n_state = 3 * self.N_fm * self.nr
        self._scalars = {}
        self.base_elems = int(L.sdd_plan_base_cache_elems(h))

    # ------------------------------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            torch = _torch()
            with torch.cuda.device(self.device):
                self._L.sdd_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------------------------------
    def _chk(self, t, n, name):
        torch = _torch()
        if not isinstance(t, torch.Tensor) or t.dtype != torch.float64 or t.device != self.device:
            raise TypeError(f"{name}: expected a float64 tensor on {self.device}")
        if not t.is_contiguous() or t.numel() % n != 0:
            raise ValueError(f"{name}: expected a contiguous tensor of batch x {n} elements")
        return t.numel() // n

    def _vec(self, v, batch):
        torch = _torch()
        if isinstance(v, torch.Tensor):
            v = v.to(device=self.device, dtype=torch.float64).reshape(-1)
            if v.numel() == 1:
                v = v.expand(batch).contiguous()
            return v.contiguous()
        # scalar parameters: one cached device vector per (value, batch), so repeated calls pass the same
        # pointers (sdd_step replays its captured graphs only for the pointers they were captured with)
        key = (float(v), int(batch))
        t = self._scalars.get(key)
        if t is None:
            if len(self._scalars) >= 64:
                self._scalars.clear()
            t = torch.full((batch,), float(v), dtype=torch.float64, device=self.device)
            self._scalars[key] = t
        return t

    def reserve(self, batch):
        """Allocate the plan's workspace for up to ``batch`` shells now (required before graph capture)."""
        torch = _torch()
        with torch.cuda.device(self.device):
            _lib.check(self._L.sdd_plan_reserve(self._h, int(batch)), "sdd_plan_reserve")

    def set_chain_layout(self, layout):
        """0 automatic, 1 one lane per row, 2 chunked (sequential carry), 3 chunked (parallel carry), 4 rows
        split over 4 warps, 5 rows split over 2 lanes in 2 warps, 6 / 7 the reference's order of operations
        without the h pre-pass, rows over 2 / 4 lanes (full right-hand sides only; otherwise 5), 8 the same
        with a (parity, shell)'s three chains in one CTA, 9 the pre-pass form with a (parity, shell)'s three
        chains in one CTA, 10 / 11 the chunks of 2 / 3 in the reference's order (FP64 right-hand sides, full
        or fused; otherwise 2 / 3) (sdd_plan_set_chain_layout); the results agree to rounding."""
        _lib.check(self._L.sdd_plan_set_chain_layout(self._h, int(layout)), "sdd_plan_set_chain_layout")
        self.chain_layout = int(layout)

    def set_chunk_length(self, chunk_set, kc):
        """Steps per chunk of chunk set 0 (layouts 2 / 10) or 1 (layouts 3 / 11); 0 restores the rule
        (sdd_plan_set_chunk_length: the set's tables are rebuilt; synchronises the device)."""
        _lib.check(self._L.sdd_plan_set_chunk_length(self._h, int(chunk_set), int(kc)), "sdd_plan_set_chunk_length")
        self.chunk_length[int(chunk_set)] = int(kc)

    def set_fx_split(self, mode):
        """0 automatic, 1 fused row kernel, 2 split row work (sdd_plan_set_fx_split); identical results."""
        _lib.check(self._L.sdd_plan_set_fx_split(self._h, int(mode)), "sdd_plan_set_fx_split")
        self.fx_split = int(mode)

    def set_tensor_cores(self, on):
        """Mixed plans: FP32 radial contractions on the tensor cores (True, the default; 3xTF32 tcgen05 products)
        or on the CUDA cores (False) (sdd_plan_set_tensor_cores)."""
        _lib.check(self._L.sdd_plan_set_tensor_cores(self._h, int(bool(on))), "sdd_plan_set_tensor_cores")
        self.tensor_cores = bool(on)

    def tensor_core_timed_out(self):
        """True if a tensor-core kernel of this plan gave up waiting for its products (sdd_plan_tensor_core_status)."""
        v = ctypes.c_int(0)
        _lib.check(self._L.sdd_plan_tensor_core_status(self._h, ctypes.byref(v)), "sdd_plan_tensor_core_status")
        return bool(v.value)

    def set_product_graphs(self, on):
        """True (the default): Newton / continuation GMRES products replay captured CUDA graphs; False: launched
        kernel by kernel, with identical results (sdd_plan_set_product_graphs)."""
        _lib.check(self._L.sdd_plan_set_product_graphs(self._h, int(bool(on))), "sdd_plan_set_product_graphs")

    def product_graph_stats(self):
        """{"captured", "replayed", "direct"}: how this plan's GMRES products ran so far
        (sdd_plan_product_graph_stats)."""
        v = [ctypes.c_longlong(0) for _ in range(3)]
        _lib.check(self._L.sdd_plan_product_graph_stats(self._h, *[ctypes.byref(x) for x in v]),
                   "sdd_plan_product_graph_stats")
        return dict(zip(("captured", "replayed", "direct"), (x.value for x in v)))

    def new_state(self, batch=1):
        torch = _torch()
        return torch.zeros((batch, self.n_state), dtype=torch.float64, device=self.device)

    def new_base(self, batch=1):
        torch = _torch()
        return torch.empty((batch, self.base_elems), dtype=torch.float64, device=self.device)

    # ---- entry points -------------------------------------------------------------------------
    def nlin_fx(self, X, out=None, base=None):
        B = self._chk(X, self.n_state, "X")
        out = out if out is not None else _torch().empty_like(X)
        _lib.check(self._L.sdd_nlin_fx(self._h, B, _dptr(X), _dptr(out), _dptr(base), _stream(self.device)),
                   "sdd_nlin_fx")
        return out

    def nlin_dfx(self, dv, X=None, base=None, out=None):
        B = self._chk(dv, self.n_state, "dv")
        out = out if out is not None else _torch().empty_like(dv)
        _lib.check(self._L.sdd_nlin_dfx(self._h, B, _dptr(dv), _dptr(X), _dptr(base), _dptr(out),
                                        _stream(self.device)), "sdd_nlin_dfx")
        return out

    def a4_bsub(self, g, out=None):
        B = self._chk(g, self.N_fm * self.nr, "g")
        out = out if out is not None else _torch().empty_like(g)
        _lib.check(self._L.sdd_a4_bsub(self._h, B, _dptr(g), _dptr(out), _stream(self.device)), "sdd_a4_bsub")
        return out

    def nab2_bsub(self, field, g, out=None):
        B = self._chk(g, self.N_fm * self.nr, "g")
        out = out if out is not None else _torch().empty_like(g)
        _lib.check(self._L.sdd_nab2_bsub(self._h, int(field), B, _dptr(g), _dptr(out), _stream(self.device)),
                   "sdd_nab2_bsub")
        return out

    def theta_op(self, op, g, out=None):
        B = self._chk(g, self.N_fm * self.nr, "g")
        out = out if out is not None else _torch().empty_like(g)
        _lib.check(self._L.sdd_theta_op(self._h, int(op), B, _dptr(g), _dptr(out), _stream(self.device)),
                   "sdd_theta_op")
        return out

    def step(self, X, Ra, Ra_s, nsteps=1, linear=False, out=None):
        B = self._chk(X, self.n_state, "X")
        out = out if out is not None else _torch().empty_like(X)
        ra, ras = self._vec(Ra, B), self._vec(Ra_s, B)
        _lib.check(self._L.sdd_step(self._h, B, _dptr(ra), _dptr(ras), _dptr(X), _dptr(out), int(nsteps),
                                    int(bool(linear)), _stream(self.device)), "sdd_step")
        return out

    def step_cnab2(self, X, Ra, Ra_s, hist, hist_valid, out=None):
        """One Crank-Nicolson / Adams-Bashforth-2 step of dt = 2 * self.dt (the plan holds the operators of
        the half step; sdd_step_cnab2).  hist: device tensor like X holding the previous step's explicit terms
        when hist_valid, overwritten with this step's.  Returns the new state."""
        B = self._chk(X, self.n_state, "X")
        self._chk(hist, self.n_state, "hist")
        out = out if out is not None else _torch().empty_like(X)
        ra, ras = self._vec(Ra, B), self._vec(Ra_s, B)
        _lib.check(self._L.sdd_step_cnab2(self._h, B, _dptr(ra), _dptr(ras), _dptr(X), _dptr(out), _dptr(hist),
                                          int(bool(hist_valid)), _stream(self.device)), "sdd_step_cnab2")
        return out

    def pfx(self, X, Ra, Ra_s, out=None, base=None):
        B = self._chk(X, self.n_state, "X")
        out = out if out is not None else _torch().empty_like(X)
        ra, ras = self._vec(Ra, B), self._vec(Ra_s, B)
        _lib.check(self._L.sdd_pfx(self._h, B, _dptr(ra), _dptr(ras), _dptr(X), _dptr(out), _dptr(base),
                                   _stream(self.device)), "sdd_pfx")
        return out

    def pdfx(self, dv, X, Ra, Ra_s, base=None, out=None):
        B = self._chk(dv, self.n_state, "dv")
        out = out if out is not None else _torch().empty_like(dv)
        ra, ras = self._vec(Ra, B), self._vec(Ra_s, B)
        _lib.check(self._L.sdd_pdfx(self._h, B, _dptr(ra), _dptr(ras), _dptr(dv), _dptr(X), _dptr(base),
                                    _dptr(out), _stream(self.device)), "sdd_pdfx")
        return out


    def deriv_tc(self, X32, out=None):
        """The four radial contractions of every mode (Dr psi, (D^2/r^2) psi, Dr T, Dr S) of a batch of FP32
        states on the tensor cores (sdd_deriv_tc, mixed plans): (batch, 4, nr, N_fm) float32."""
        torch = _torch()
        if not isinstance(X32, torch.Tensor) or X32.dtype != torch.float32 or X32.device != self.device or \
                not X32.is_contiguous() or X32.numel() % self.n_state:
            raise TypeError("X32: expected a contiguous float32 tensor of batch x n_state on the plan's device")
        B = X32.numel() // self.n_state
        if out is None:
            out = torch.empty((B, 4, self.nr, self.N_fm), dtype=torch.float32, device=self.device)
        _lib.check(self._L.sdd_deriv_tc(self._h, B, _dptr(X32), _dptr(out), _stream(self.device)), "sdd_deriv_tc")
        return out

    def step_profile(self, X, Ra, Ra_s, nsteps):
        """Per-kernel milliseconds (fx, rhs, chain) summed over nsteps steps from X (CUDA events)."""
        B = self._chk(X, self.n_state, "X")
        ra, ras = self._vec(Ra, B), self._vec(Ra_s, B)
        out = _torch().empty_like(X)
        ms = (ctypes.c_double * 3)(0.0, 0.0, 0.0)
        _lib.check(self._L.sdd_step_profile(self._h, B, _dptr(ra), _dptr(ras), _dptr(X), _dptr(out), int(nsteps),
                                            ms, _stream(self.device)), "sdd_step_profile")
        return list(ms), out

    def diagnostics(self, X):
        """(batch, 4) device tensor: |X|_2, Kinetic_Energy, Nusselt(T), Nusselt(S) of each shell
        (Main.py:41-134, sdd_diagnostics)."""
        torch = _torch()
        B = self._chk(X, self.n_state, "X")
        out = torch.empty((B, 4), dtype=torch.float64, device=self.device)
        _lib.check(self._L.sdd_diagnostics(self._h, B, _dptr(X), _dptr(out), _stream(self.device)), "sdd_diagnostics")
        return out

    def step_diag(self, X, Ra, Ra_s, nsteps=1, linear=False, out=None):
        """nsteps steps like ``step`` with the diagnostics of the state after every step:
        returns (X_out, (nsteps, batch, 4) device tensor)."""
        torch = _torch()
        B = self._chk(X, self.n_state, "X")
        out = out if out is not None else torch.empty_like(X)
        ra, ras = self._vec(Ra, B), self._vec(Ra_s, B)
        dg = torch.empty((max(int(nsteps), 0), B, 4), dtype=torch.float64, device=self.device)
        _lib.check(self._L.sdd_step_diag(self._h, B, _dptr(ra), _dptr(ras), _dptr(X), _dptr(out), int(nsteps),
                                         int(bool(linear)), _dptr(dg), _stream(self.device)), "sdd_step_diag")
        return out, dg

    def chain_choice(self, batch=1):
        """(layout, kc, nch) that a step of ``batch`` shells runs its chains with (sdd_plan_chain_choice)."""
        lay, kc, nch = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _lib.check(self._L.sdd_plan_chain_choice(self._h, int(batch), ctypes.byref(lay), ctypes.byref(kc),
                                                 ctypes.byref(nch)), "sdd_plan_chain_choice")
        return lay.value, kc.value, nch.value

    def chunks(self, batch=1):
        """Chunks per chain of the chains a step of ``batch`` shells runs (1 when not chunked)."""
        return self.chain_choice(batch)[2]

    def kernel_profile(self, X, Ra, Ra_s, nsteps):
        """{kernel name: (total milliseconds, launches)} over nsteps steps from X, with a CUDA event after
        every kernel launch (sdd_step_kernel_profile); kernels that did not run are left out."""
        B = self._chk(X, self.n_state, "X")
        ra, ras = self._vec(Ra, B), self._vec(Ra_s, B)
        out = _torch().empty_like(X)
        n = 10                         # SDD_NUM_KERNELS
        ms = (ctypes.c_double * n)(*([0.0] * n))
        cnt = (ctypes.c_int * n)(*([0] * n))
        _lib.check(self._L.sdd_step_kernel_profile(self._h, B, _dptr(ra), _dptr(ras), _dptr(X), _dptr(out),
                                                   int(nsteps), ms, cnt, _stream(self.device)),
                   "sdd_step_kernel_profile")
        return {self._L.sdd_kernel_name(k).decode(): (ms[k], cnt[k]) for k in range(n) if cnt[k] > 0}

    def newton(self, X, Ra, Ra_s, tol=1e-10, restart=50, gmres_rtol=1e-4, max_newton=20, max_restarts=20,
               mixed_matvec=False, raise_on_fail=False):
        """Newton-GMRES on F(X) = Phi_dt(X) - X in place on X (batch x n_state); returns per-shell dicts
        (residual0, residual, newton_iters, matvecs, converged).  The plan's dt should be 1 (Main.py:430).
        mixed_matvec (mixed plans): False/0 FP64 Jacobian products, True/1 with the FP32 nonlinear term,
        2 also with FP32 right-hand sides and h = Linv g matvecs (the chains and the residual stay FP64),
        3 as 2 with the GMRES basis stored and orthogonalised in FP32 (the Newton residual stays FP64)."""
        B = self._chk(X, self.n_state, "X")
        ra, ras = self._vec(Ra, B), self._vec(Ra_s, B)
        mv = int(mixed_matvec)
        if mv not in (0, 1, 2, 3):
            raise ValueError("mixed_matvec: expected False/True, 0, 1, 2 or 3")
        o = _lib.NewtonOpts(float(tol), float(gmres_rtol), int(restart), int(max_restarts), int(max_newton), mv)
        res = (_lib.NewtonResult * B)()
        st = self._L.sdd_newton_gmres(self._h, B, _dptr(ra), _dptr(ras), _dptr(X), ctypes.byref(o), res,
                                      _stream(self.device))
        if st not in (_lib.SDD_OK, _lib.SDD_ERR_NOT_CONVERGED) or (raise_on_fail and st != _lib.SDD_OK):
            _lib.check(st, "sdd_newton_gmres")
        return [dict(residual0=r.residual0, residual=r.residual, newton_iters=r.newton_iters,
                     matvecs=r.matvecs, converged=bool(r.converged)) for r in res]


    def set_reorth_eta(self, eta):
        """GMRES: repeat a column's Gram-Schmidt pass where the first left |w'| < eta |w| (default 1/sqrt(2))."""
        _lib.check(self._L.sdd_plan_set_reorth_eta(self._h, float(eta)), "sdd_plan_set_reorth_eta")

    def krylov_basis(self, shell, max_cols=64):
        """(k x n_state) device tensor: the basis vectors of the last GMRES cycle of the last solve for one
        shell (sdd_krylov_basis)."""
        torch = _torch()
        out = torch.empty((max_cols, self.n_state), dtype=torch.float64, device=self.device)
        k = ctypes.c_int(0)
        _lib.check(self._L.sdd_krylov_basis(self._h, int(shell), int(max_cols), _dptr(out), ctypes.byref(k),
                                            _stream(self.device)), "sdd_krylov_basis")
        return out[:k.value]

    def contin_step(self, X, Ra, Ra_s, sign, ds, tol=1e-10, restart=50, gmres_rtol=1e-4, tangent_rtol=1e-8,
                    max_restarts=20, max_corrector=5, max_halvings=8, mixed_matvec=False):
        """One pseudo-arclength step (sdd_contin_step) in place on X (batch x n_state) and Ra (device,
        batch).  mixed_matvec as in ``newton`` (mixed plans).  Returns (X_dot tensor, per-shell result
        dicts)."""
        torch = _torch()
        B = self._chk(X, self.n_state, "X")
        if not (isinstance(Ra, torch.Tensor) and Ra.dtype == torch.float64 and Ra.device == self.device
                and Ra.numel() == B and Ra.is_contiguous()):
            raise TypeError("Ra: expected a contiguous float64 device tensor with one entry per shell")
        ras = self._vec(Ra_s, B)
        Xd = torch.empty_like(X)
        sg = (ctypes.c_double * B)(*[float(v) for v in np.broadcast_to(np.asarray(sign, dtype=float), (B,))])
        dd = (ctypes.c_double * B)(*[float(v) for v in np.broadcast_to(np.asarray(ds, dtype=float), (B,))])
        mv = int(mixed_matvec)
        if mv not in (0, 1, 2, 3):
            raise ValueError("mixed_matvec: expected False/True, 0, 1, 2 or 3")
        o = _lib.ContinOpts(float(tol), float(gmres_rtol), float(tangent_rtol), int(restart), int(max_restarts),
                            int(max_corrector), int(max_halvings), mv, 0)
        res = (_lib.ContinResult * B)()
        st = self._L.sdd_contin_step(self._h, B, _dptr(X), _dptr(Ra), _dptr(ras), _dptr(Xd), sg, dd,
                                     ctypes.byref(o), res, _stream(self.device))
        if st not in (_lib.SDD_OK, _lib.SDD_ERR_NOT_CONVERGED):
            _lib.check(st, "sdd_contin_step")
        return Xd, [dict(residual=r.residual, arclength=r.arclength, ds=r.ds, Ra_dot=r.Ra_dot,
                         corrector_iters=r.corrector_iters, halvings=r.halvings, matvecs=r.matvecs,
                         converged=bool(r.converged)) for r in res]


def batch_step(groups, nsteps=1, linear=False):
    """Advance several plans' shells at once (sdd_batch_step): ``groups`` is a list of (plan, X, Ra, Ra_s) or
    (plan, X, Ra, Ra_s, out) with X a (shells x n_state) device tensor of that plan, one entry per distinct
    plan, all on one device.  Every group runs sdd_step on its plan's own branch stream, forked from and joined
    back into the current stream, so the groups run concurrently; each group's result equals its
    ``plan.step`` alone.  Returns the output tensors in the order of ``groups``."""
    torch = _torch()
    if not groups:
        raise ValueError("batch_step: no groups")
    dev = groups[0][0].device
    arr = (_lib.BatchGroup * len(groups))()
    outs, keep = [], []
    for k, g in enumerate(groups):
        plan, X, Ra, Ra_s = g[:4]
        if plan.device != dev:
            raise ValueError("batch_step: every plan must be on one device")
        B = plan._chk(X, plan.n_state, "X")
        out = g[4] if len(g) > 4 and g[4] is not None else torch.empty_like(X)
        plan._chk(out, plan.n_state, "out")
        ra, ras = plan._vec(Ra, B), plan._vec(Ra_s, B)
        keep += [ra, ras]
        arr[k] = _lib.BatchGroup(plan._h.value, B, 0, ra.data_ptr(), ras.data_ptr(), X.data_ptr(), out.data_ptr())
        outs.append(out)
    L = groups[0][0]._L
    _lib.check(L.sdd_batch_step(arr, len(groups), int(nsteps), int(bool(linear)), _stream(dev)), "sdd_batch_step")
    return outs


_cache = {}
_cache_lock = threading.Lock()


def get_plan(N_fm, N_r, d, dt, Pr, Tau, symmetric=False, precision="fp64", device=None):
    """Cached plan for the key (N_fm, N_r, d, dt, Pr, Tau, symmetric, precision, device)."""
    torch = _torch()
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    key = (int(N_fm), int(N_r), float(d), float(dt), float(Pr), float(Tau), bool(symmetric), precision, str(dev))
    with _cache_lock:
        p = _cache.get(key)
        if p is None:
            p = Plan(N_fm, N_r, d, dt, Pr, Tau, symmetric, precision, dev)
            _cache[key] = p
        return p


def clear_plans():
    with _cache_lock:
        for p in _cache.values():
            p.close()
        _cache.clear()


class CNAB2Stepper:
    """Crank-Nicolson (implicit terms) / Adams-Bashforth 2 (explicit terms) time stepping of a batch of
    shells: an opt-in, second-order scheme beside the reference's IMEX Euler ("CNAB1", Main.py:255-283,
    which Plan.step reproduces).  The first step's explicit part is Euler; the explicit terms of the last
    step are kept on the device for the next.  Uses a plan of dt/2 (sdd_step_cnab2)."""

    def __init__(self, N_fm, N_r, d, dt, Pr, Tau, symmetric=False, precision="fp64", device=None):
        self.plan = Plan(N_fm, N_r, d, 0.5 * float(dt), Pr, Tau, symmetric=symmetric, precision=precision,
                         device=device)
        self.dt = float(dt)
        self.hist = None
        self.valid = False

    def reset(self):
        self.valid = False

    def step(self, X, Ra, Ra_s, nsteps=1):
        torch = _torch()
        if self.hist is None or self.hist.shape != X.shape:
            self.hist = torch.empty_like(X)
            self.valid = False
        a, b = X, torch.empty_like(X)
        for _ in range(int(nsteps)):
            self.plan.step_cnab2(a, Ra, Ra_s, self.hist, self.valid, out=b)
            self.valid = True
            a, b = b, (a if a is not X else torch.empty_like(X))
        return a
