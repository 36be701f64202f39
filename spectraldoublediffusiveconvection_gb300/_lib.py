"""ctypes binding of ``libsdd_gb300.so`` (the C ABI declared in ``include/sdd_gb300.h``).

There is no CPU fallback: importing a compute entry point without the built library raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsdd_gb300.so")

SDD_OK = 0
SDD_ERR_ARG = -1
SDD_ERR_ODD_NFM = -2
SDD_ERR_UNSUPPORTED = -3
SDD_ERR_CUDA = -4
SDD_ERR_NOMEM = -5
SDD_ERR_NOT_CONVERGED = -6

SDD_PREC_FP64 = 0
SDD_PREC_MIXED = 1

SDD_IDCT, SDD_IDST, SDD_DCT, SDD_DST = 0, 1, 2, 3

SDD_NOALLOC_SCRATCH_DOUBLES = 1 << 20

_dp = ctypes.POINTER(ctypes.c_double)


class PlanDesc(ctypes.Structure):
    """Mirror of ``sdd_plan_desc``."""
    _fields_ = [
        ("N_fm", ctypes.c_int32), ("nr", ctypes.c_int32), ("symmetric", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("dt", ctypes.c_double), ("Pr", ctypes.c_double), ("Tau", ctypes.c_double),
        ("Dr", _dp), ("D2_r2", _dp), ("ir4_r2", _dp), ("D2_sine", _dp), ("ir2_sine", _dp),
        ("D2_A4", _dp), ("ir2_A4", _dp), ("ir4_A4", _dp), ("rsq", _dp), ("dT0", _dp), ("gr", _dp),
        ("Linv_A4", _dp), ("Linv_T", _dp), ("Linv_S", _dp),
        ("nu_w", _dp), ("r_int", _dp), ("r_i", ctypes.c_double), ("r_o", ctypes.c_double),
    ]


class NewtonOpts(ctypes.Structure):
    """Mirror of ``sdd_newton_opts``."""
    _fields_ = [("tol", ctypes.c_double), ("gmres_rtol", ctypes.c_double), ("restart", ctypes.c_int32),
                ("max_restarts", ctypes.c_int32), ("max_newton", ctypes.c_int32),
                ("mixed_matvec", ctypes.c_int32)]


class NewtonResult(ctypes.Structure):
    """Mirror of ``sdd_newton_result``."""
    _fields_ = [("residual0", ctypes.c_double), ("residual", ctypes.c_double),
                ("newton_iters", ctypes.c_int32), ("matvecs", ctypes.c_int32),
                ("converged", ctypes.c_int32), ("pad", ctypes.c_int32)]


class ContinOpts(ctypes.Structure):
    """Mirror of ``sdd_contin_opts``."""
    _fields_ = [("tol", ctypes.c_double), ("gmres_rtol", ctypes.c_double), ("tangent_rtol", ctypes.c_double),
                ("restart", ctypes.c_int32), ("max_restarts", ctypes.c_int32), ("max_corrector", ctypes.c_int32),
                ("max_halvings", ctypes.c_int32), ("mixed_matvec", ctypes.c_int32), ("pad", ctypes.c_int32)]


class ContinResult(ctypes.Structure):
    """Mirror of ``sdd_contin_result``."""
    _fields_ = [("residual", ctypes.c_double), ("arclength", ctypes.c_double), ("ds", ctypes.c_double),
                ("Ra_dot", ctypes.c_double), ("corrector_iters", ctypes.c_int32), ("halvings", ctypes.c_int32),
                ("matvecs", ctypes.c_int32), ("converged", ctypes.c_int32)]


class BatchGroup(ctypes.Structure):
    """Mirror of ``sdd_batch_group``."""
    _fields_ = [("plan", ctypes.c_void_p), ("batch", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("Ra", ctypes.c_void_p), ("Ra_s", ctypes.c_void_p), ("X_in", ctypes.c_void_p),
                ("X_out", ctypes.c_void_p)]


# (name, restype, argtypes) of every exported symbol; the CPU test checks the header declares these.
_VP = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
SIGNATURES = [
    ("sdd_error_string", ctypes.c_char_p, [_I]),
    ("sdd_last_cuda_error", _I, []),
    ("sdd_version", _I, []),
    ("sdd_transform", _I, [_I, _I, _I, _I, _VP, _VP, _VP]),
    ("sdd_plan_create", _I, [ctypes.POINTER(PlanDesc), ctypes.POINTER(_VP)]),
    ("sdd_plan_destroy", _I, [_VP]),
    ("sdd_plan_reserve", _I, [_VP, _I]),
    ("sdd_plan_set_chain_layout", _I, [_VP, _I]),
    ("sdd_plan_set_fx_split", _I, [_VP, _I]),
    ("sdd_plan_set_tensor_cores", _I, [_VP, _I]),
    ("sdd_plan_tensor_core_status", _I, [_VP, ctypes.POINTER(_I)]),
    ("sdd_plan_set_product_graphs", _I, [_VP, _I]),
    ("sdd_probe_phase_boundaries", _I, [_I, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_I), _VP]),
    ("sdd_plan_product_graph_stats", _I, [_VP, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
                                          ctypes.POINTER(ctypes.c_longlong)]),
    ("sdd_plan_chain_choice", _I, [_VP, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    ("sdd_plan_base_cache_elems", ctypes.c_size_t, [_VP]),
    ("sdd_nlin_fx", _I, [_VP, _I, _VP, _VP, _VP, _VP]),
    ("sdd_nlin_dfx", _I, [_VP, _I, _VP, _VP, _VP, _VP, _VP]),
    ("sdd_a4_bsub", _I, [_VP, _I, _VP, _VP, _VP]),
    ("sdd_nab2_bsub", _I, [_VP, _I, _I, _VP, _VP, _VP]),
    ("sdd_theta_op", _I, [_VP, _I, _I, _VP, _VP, _VP]),
    ("sdd_step", _I, [_VP, _I, _VP, _VP, _VP, _VP, _I, _I, _VP]),
    ("sdd_batch_step", _I, [ctypes.POINTER(BatchGroup), _I, _I, _I, _VP]),
    ("sdd_plan_set_chunk_length", _I, [_VP, _I, _I]),
    ("sdd_step_cnab2", _I, [_VP, _I, _VP, _VP, _VP, _VP, _VP, _I, _VP]),
    ("sdd_pfx", _I, [_VP, _I, _VP, _VP, _VP, _VP, _VP, _VP]),
    ("sdd_pdfx", _I, [_VP, _I, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    ("sdd_newton_gmres", _I, [_VP, _I, _VP, _VP, _VP, ctypes.POINTER(NewtonOpts), ctypes.POINTER(NewtonResult),
                              _VP]),
    ("sdd_plan_set_reorth_eta", _I, [_VP, _D]),
    ("sdd_krylov_basis", _I, [_VP, _I, _I, _VP, ctypes.POINTER(_I), _VP]),
    ("sdd_contin_step", _I, [_VP, _I, _VP, _VP, _VP, _VP, ctypes.POINTER(ctypes.c_double),
                             ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ContinOpts),
                             ctypes.POINTER(ContinResult), _VP]),
    ("sdd_nlin_fx_noalloc", _I, [_VP, _I, _VP, _VP, _VP]),
    ("sdd_deriv_tc", _I, [_VP, _I, _VP, _VP, _VP]),
    ("sdd_step_profile", _I, [_VP, _I, _VP, _VP, _VP, _VP, _I, ctypes.POINTER(ctypes.c_double), _VP]),
    ("sdd_diagnostics", _I, [_VP, _I, _VP, _VP, _VP]),
    ("sdd_step_diag", _I, [_VP, _I, _VP, _VP, _VP, _VP, _I, _I, _VP, _VP]),
    ("sdd_kernel_name", ctypes.c_char_p, [_I]),
    ("sdd_step_kernel_profile", _I, [_VP, _I, _VP, _VP, _VP, _VP, _I, ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(ctypes.c_int), _VP]),
    ("sdd_measure_fp64_peak", _I, [ctypes.POINTER(ctypes.c_double), _VP]),
    ("sdd_debug_fail_allocations", _I, [ctypes.c_longlong]),
]

_lib = None


class SDDError(RuntimeError):
    """A non-zero status from libsdd_gb300."""

    def __init__(self, status, where):
        self.status = status
        msg = lib().sdd_error_string(status).decode()
        if status == SDD_ERR_CUDA:
            msg += f" (cudaError {lib().sdd_last_cuda_error()})"
        super().__init__(f"{where}: {msg} [status {status}]")


class SDDMemoryError(SDDError, MemoryError):
    """SDD_ERR_NOMEM: a device allocation of the library failed."""


def load(path=LIB_PATH):
    """Load the shared library (no CUDA context is created by loading)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build it with `python -m spectraldoublediffusiveconvection_gb300.build`"
            " (there is no CPU fallback)")
    L = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def lib():
    return _lib if _lib is not None else load()


def check(status, where):
    if status != SDD_OK:
        if status == SDD_ERR_ODD_NFM:
            raise ValueError(f"The number of Fourier modes is not even ({where})")
        if status == SDD_ERR_NOMEM:
            raise SDDMemoryError(status, where)
        raise SDDError(status, where)
    return status
