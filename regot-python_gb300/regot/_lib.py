"""Loader and ctypes declarations of libregot_gb300.so (include/regot_gb300.h).

The library is built in-tree by ``regot-python_gb300/build.py`` (called from
``__graft_entry__.build()``). There is no CPU fallback: importing a solver
without the compiled library raises ImportError, and calling one without a
CUDA device raises RuntimeError.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
import weakref

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "_build", "libregot_gb300.so")

REGOT_OK = 0
REGOT_ERR_INVALID_ARG = 1
REGOT_ERR_NO_DEVICE = 7
REGOT_ERR_TOO_LARGE = 8
REGOT_F64, REGOT_F32 = 0, 1
REGOT_MEM_HOST, REGOT_MEM_DEVICE = 0, 1
REGOT_PREC_FP64, REGOT_PREC_MIXED = 0, 1

_dp = C.POINTER(C.c_double)


class ProblemDesc(C.Structure):
    _fields_ = [
        ("M", C.c_void_p),
        ("M_dtype", C.c_int),
        ("M_mem", C.c_int),
        ("ldm", C.c_longlong),
        ("n", C.c_int),
        ("m", C.c_int),
        ("a", C.c_void_p),
        ("b", C.c_void_p),
        ("ab_mem", C.c_int),
    ]


class Opts(C.Structure):
    _fields_ = [
        ("precision", C.c_int),
        ("method", C.c_int),
        ("mu0", C.c_double),
        ("shift", C.c_double),
        ("density", C.c_double),
        ("tau", C.c_double),
        ("x0", _dp),
        ("x0_len", C.c_int),
        ("cg_tol", C.c_double),
        ("cg_max_iter", C.c_int),
        ("verbose", C.c_int),
        ("plan", C.c_int),
        ("plan_mem", C.c_int),
        ("prim_vals", C.c_int),
    ]


class Result(C.Structure):
    _fields_ = [
        ("niter", C.c_int),
        ("hist_len", C.c_int),
        ("hist_cap", C.c_int),
        ("dual", C.c_void_p),
        ("plan", C.c_void_p),
        ("obj_vals", C.c_void_p),
        ("mar_errs", C.c_void_p),
        ("run_times", C.c_void_p),
        ("densities", C.c_void_p),
        ("prim_vals", C.c_void_p),
        ("passes", C.c_longlong),
        ("solve_ms", C.c_double),
    ]


class PdipOpts(C.Structure):
    _fields_ = [
        ("inner_solver", C.c_int),
        ("cg_max_iter", C.c_int),
        ("fixed_threshold", C.c_double),
        ("fp_max_iter", C.c_int),
        ("fp_exit_scale", C.c_double),
        ("fp_stop_gap_mu_only", C.c_int),
        ("cg_stop_gap_mu_only", C.c_int),
        ("cg_mar_tol", C.c_double),
    ]


class BatchDesc(C.Structure):
    _fields_ = [
        ("count", C.c_int),
        ("n", C.c_void_p),
        ("m", C.c_void_p),
        ("d", C.c_void_p),
        ("cost_scale", C.c_void_p),
        ("x", C.c_void_p),
        ("y", C.c_void_p),
        ("a", C.c_void_p),
        ("b", C.c_void_p),
        ("mem", C.c_int),
    ]


class BatchResult(C.Structure):
    _fields_ = [
        ("alpha", C.c_void_p),
        ("beta", C.c_void_p),
        ("niter", C.c_void_p),
        ("mar_err", C.c_void_p),
        ("sweeps", C.c_longlong),
        ("solve_ms", C.c_double),
    ]


BATCH_MAX_DIM = 16

# Dense pass kinds of regot_time_pass / regot_pass_bytes (REGOT_PASS_*), with
# the name of the kernel instance each one launches.
PASS_KINDS = [
    ("EROT_ROW", "OP_E_ROW"), ("EROT_COL", "OP_E_COL"), ("EROT_GRAD", "OP_E_ROWCOL"),
    ("EROT_HVP", "OP_E_HVP"), ("QROT_GRAD", "OP_Q_GRAD"), ("EROT_LS", "OP_E_LS"),
    ("EROT_GRADLS", "OP_E_GRADLS"), ("EROT_AVG", "OP_E_AVG"), ("EROT_PLAN", "OP_E_PLAN"),
    ("EROT_ROWMAX", "OP_E_ROWMAX"), ("EROT_COLMAX", "OP_E_COLMAX"),
    ("QROT_GRADMASK", "OP_Q_GRADMASK"), ("QROT_GRADLS", "OP_Q_GRADLS"), ("QROT_OBJ", "OP_Q_OBJ"),
    ("QROT_P1", "OP_Q_P1"), ("QROT_P2", "OP_Q_P2"), ("QROT_P3", "OP_Q_P3"),
    ("QROT_COLROOT", "OP_Q_COLROOT"), ("QROT_ROWROOT", "OP_Q_ROWROOT"), ("QROT_AVG", "OP_Q_AVG"),
    ("QROT_PLAN", "OP_Q_PLAN"),
]


# Every symbol include/regot_gb300.h declares.
EXPORTS = [
    "regot_opts_init", "regot_ctx_create", "regot_ctx_destroy", "regot_ctx_last_error",
    "regot_ctx_set_stream", "regot_ctx_own_stream", "regot_ctx_kernel_launches", "regot_problem_create",
    "regot_problem_destroy", "regot_sinkhorn_bcd", "regot_sinkhorn_newton",
    "regot_sinkhorn_ssns", "regot_sinkhorn_lbfgs_dual", "regot_sinkhorn_apdagd",
    "regot_sinkhorn_sparse_newton", "regot_sinkhorn_splr",
    "regot_qrot_lbfgs_dual", "regot_qrot_assn", "regot_qrot_bcd", "regot_qrot_gd",
    "regot_qrot_apdagd", "regot_qrot_pdaam", "regot_qrot_grssn", "regot_qrot_lbfgs_semi_dual",
    "regot_qrot_optimal_alpha", "regot_qrot_pdip", "regot_pdip_opts_init", "regot_erot_optimal_beta", "regot_erot_optimal_alpha", "regot_erot_dual_obj_grad",
    "regot_erot_hvp", "regot_erot_plan", "regot_erot_sparsify", "regot_erot_sparsify_density",
    "regot_erot_hess_solve",
    "regot_erot_tyy", "regot_erot_tty", "regot_sqeuclid_cost", "regot_erot_solve_batched", "regot_erot_solve_batched_grad",
    "regot_qrot_dual_obj_grad",
    "regot_qrot_optimal_beta",
    "regot_qrot_primal_val", "regot_qrot_plan", "regot_time_pass", "regot_pass_bytes",
    "regot_set_wait_limit", "regot_autotune", "regot_autotune_save", "regot_autotune_load",
    "regot_autotune_clear", "regot_autotune_entries", "regot_force_pass_config",
    "regot_pass_config", "regot_force_batch_variant", "regot_batch_variants",
    "regot_force_sparsify_path",
    "regot_force_qrot_cg_path", "regot_set_batch_tail",
    "regot_erot_dual_obj_grad_noalloc", "regot_host_alloc", "regot_host_free",
]

_lib = None
_lock = threading.Lock()


def load() -> C.CDLL:
    """Load the shared library (once) and declare the signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing; build it with "
                "`python regot-python_gb300/build.py` (needs nvcc)")
        lib = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        lib.regot_opts_init.argtypes = [C.POINTER(Opts)]
        lib.regot_opts_init.restype = None
        lib.regot_ctx_create.argtypes = [C.c_int, C.POINTER(vp)]
        lib.regot_ctx_destroy.argtypes = [vp]
        lib.regot_ctx_destroy.restype = None
        lib.regot_ctx_last_error.argtypes = [vp]
        lib.regot_ctx_last_error.restype = C.c_char_p
        lib.regot_ctx_set_stream.argtypes = [vp, vp]
        lib.regot_ctx_own_stream.argtypes = [vp]
        lib.regot_ctx_own_stream.restype = vp
        lib.regot_ctx_kernel_launches.argtypes = [vp]
        lib.regot_ctx_kernel_launches.restype = C.c_longlong
        lib.regot_problem_create.argtypes = [vp, C.POINTER(ProblemDesc), C.c_int, C.POINTER(vp)]
        lib.regot_problem_destroy.argtypes = [vp]
        lib.regot_problem_destroy.restype = None
        for name in ("regot_sinkhorn_bcd", "regot_sinkhorn_newton", "regot_sinkhorn_ssns",
                     "regot_sinkhorn_sparse_newton", "regot_sinkhorn_splr",
                     "regot_sinkhorn_lbfgs_dual", "regot_sinkhorn_apdagd",
                     "regot_qrot_lbfgs_dual", "regot_qrot_assn", "regot_qrot_bcd",
                     "regot_qrot_gd", "regot_qrot_apdagd", "regot_qrot_pdaam",
                     "regot_qrot_grssn", "regot_qrot_lbfgs_semi_dual"):
            f = getattr(lib, name)
            f.argtypes = [vp, vp, C.c_double, C.c_double, C.c_int, C.POINTER(Opts),
                          C.POINTER(Result)]
        lib.regot_erot_optimal_beta.argtypes = [vp, vp, C.c_double, vp, vp]
        lib.regot_erot_optimal_alpha.argtypes = [vp, vp, C.c_double, vp, vp]
        lib.regot_erot_dual_obj_grad.argtypes = [vp, vp, C.c_double, vp, vp, vp]
        lib.regot_erot_hvp.argtypes = [vp, vp, C.c_double, vp, vp, vp]
        lib.regot_erot_plan.argtypes = [vp, vp, C.c_double, vp, vp, C.c_int]
        lib.regot_erot_sparsify.argtypes = [vp, vp, C.c_double, vp, C.c_double, C.c_double, vp,
                                             vp]
        lib.regot_pdip_opts_init.argtypes = [C.POINTER(PdipOpts)]
        lib.regot_pdip_opts_init.restype = None
        lib.regot_qrot_pdip.argtypes = [vp, vp, C.c_double, C.c_double, C.c_int,
                                        C.POINTER(PdipOpts), C.POINTER(Opts), C.POINTER(Result),
                                        C.POINTER(C.c_int)]
        lib.regot_erot_sparsify_density.argtypes = [vp, vp, C.c_double, vp, C.c_double, vp, vp]
        lib.regot_qrot_dual_obj_grad.argtypes = [vp, vp, C.c_double, vp, vp, vp]
        lib.regot_qrot_optimal_beta.argtypes = [vp, vp, C.c_double, vp, vp]
        lib.regot_qrot_primal_val.argtypes = [vp, vp, C.c_double, vp, vp]
        lib.regot_qrot_plan.argtypes = [vp, vp, C.c_double, vp, vp, C.c_int]
        lib.regot_qrot_optimal_alpha.argtypes = [vp, vp, C.c_double, vp, vp]
        lib.regot_time_pass.argtypes = [vp, vp, C.c_int, C.c_double, C.c_int]
        lib.regot_pass_bytes.argtypes = [vp, C.c_int]
        lib.regot_pass_bytes.restype = C.c_longlong
        lib.regot_set_wait_limit.argtypes = [C.c_longlong]
        lib.regot_set_wait_limit.restype = C.c_longlong
        lib.regot_autotune.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
        lib.regot_autotune_save.argtypes = [C.c_char_p]
        lib.regot_autotune_load.argtypes = [C.c_char_p]
        lib.regot_autotune_clear.argtypes = []
        lib.regot_autotune_clear.restype = None
        lib.regot_autotune_entries.argtypes = [C.c_char_p, C.c_size_t]
        lib.regot_autotune_entries.restype = C.c_size_t
        lib.regot_force_pass_config.argtypes = [C.c_int]
        lib.regot_pass_config.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
        lib.regot_force_batch_variant.argtypes = [C.c_int]
        lib.regot_force_sparsify_path.argtypes = [C.c_int]
        lib.regot_force_qrot_cg_path.argtypes = [C.c_int]
        lib.regot_set_batch_tail.argtypes = [C.c_int]
        lib.regot_batch_variants.argtypes = [vp, C.POINTER(C.c_int)]
        lib.regot_erot_solve_batched.argtypes = [vp, C.POINTER(BatchDesc), C.c_double,
                                                 C.c_double, C.c_int, C.POINTER(BatchResult)]
        lib.regot_erot_solve_batched_grad.argtypes = [vp, C.POINTER(BatchDesc), C.c_double,
                                                      C.c_double, C.c_int,
                                                      C.POINTER(BatchResult), vp, vp, vp]
        lib.regot_erot_hess_solve.argtypes = [vp, vp, C.c_double, vp, vp, C.c_double, C.c_int,
                                              vp, C.POINTER(C.c_int)]
        lib.regot_erot_tyy.argtypes = [vp, vp, C.c_double, vp, vp, vp, vp, C.c_int, vp, vp,
                                       C.c_int]
        lib.regot_erot_tty.argtypes = [vp, vp, C.c_double, vp, vp, vp, vp, C.c_int, vp, vp,
                                       C.c_int]
        lib.regot_sqeuclid_cost.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_double,
                                            C.c_int, vp, C.c_longlong]
        lib.regot_erot_dual_obj_grad_noalloc.argtypes = [
            vp, C.c_longlong, C.c_int, C.c_int, vp, vp, vp, C.c_double, vp, vp, vp]
        lib.regot_host_alloc.argtypes = [C.c_size_t, C.POINTER(vp)]
        lib.regot_host_free.argtypes = [vp]
        lib.regot_host_free.restype = None
        _lib = lib
        return lib


class Context:
    """One CUDA device and stream (regot_ctx)."""

    def __init__(self, device: int = 0):
        lib = load()
        h = C.c_void_p()
        rc = lib.regot_ctx_create(int(device), C.byref(h))
        if rc == REGOT_ERR_NO_DEVICE:
            raise RuntimeError("regot_gb300 needs a CUDA device; none is visible")
        if rc != REGOT_OK:
            raise RuntimeError(f"regot_ctx_create failed with status {rc}")
        self.handle = h
        self.device = device
        self._lib = lib

    def check(self, rc: int):
        if rc == REGOT_OK:
            return
        msg = self._lib.regot_ctx_last_error(self.handle).decode(errors="replace")
        if rc == REGOT_ERR_INVALID_ARG:
            raise ValueError(msg)
        raise RuntimeError(msg)

    def kernel_launches(self) -> int:
        return int(self._lib.regot_ctx_kernel_launches(self.handle))

    def set_stream(self, stream_ptr: int | None):
        """Launch on this cudaStream_t (0 = legacy default stream); None
        restores the context's own stream."""
        if stream_ptr is None:
            stream_ptr = self._lib.regot_ctx_own_stream(self.handle)
        self.check(self._lib.regot_ctx_set_stream(self.handle, C.c_void_p(stream_ptr or 0)))

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self._lib.regot_ctx_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


def autotune_entries() -> list[list[str]]:
    """The autotuner's table: one list of fields per entry (device,
    precision, pass, size class, configuration, microseconds of each
    configuration)."""
    lib = load()
    size = lib.regot_autotune_entries(None, 0)
    buf = C.create_string_buffer(size + 1)
    lib.regot_autotune_entries(buf, size + 1)
    return [ln.split("\t") for ln in buf.value.decode().splitlines() if ln]


_contexts: dict[int, Context] = {}


def context(device: int = 0) -> Context:
    with _lock:
        ctx = _contexts.get(device)
    if ctx is None:
        ctx = Context(device)
        with _lock:
            _contexts[device] = ctx
    return ctx


# Results at least this large go to page-locked memory.
PINNED_MIN_BYTES = 1 << 20


def host_empty(shape, dtype=np.float64) -> np.ndarray:
    """numpy array in page-locked host memory (regot_host_alloc) for large
    device-to-host results; the block returns to the library's cache when the
    last view of the array is gone. Small arrays are ordinary numpy arrays."""
    dtype = np.dtype(dtype)
    count = int(np.prod(shape))
    nbytes = count * dtype.itemsize
    if nbytes < PINNED_MIN_BYTES:
        return np.empty(shape, dtype=dtype)
    lib = load()
    ptr = C.c_void_p()
    if lib.regot_host_alloc(nbytes, C.byref(ptr)) != REGOT_OK:
        return np.empty(shape, dtype=dtype)
    buf = (C.c_byte * nbytes).from_address(ptr.value)
    weakref.finalize(buf, lib.regot_host_free, C.c_void_p(ptr.value))
    return np.frombuffer(buf, dtype=dtype, count=count).reshape(shape)
