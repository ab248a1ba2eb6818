"""ctypes binding of libgbtn.so (the C ABI declared in include/gbtn.h).

The library is required: importing :mod:`gbtn` succeeds without it, but the
first call that needs the GPU raises :class:`LibraryNotBuilt` -- there is no
CPU fallback."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np

from .build import INCLUDE, LIB_PATH

GBTN_OK = 0
ERRORS = {
    1: "GBTN_ERR_INVALID",
    2: "GBTN_ERR_CUDA",
    3: "GBTN_ERR_UNSUPPORTED",
    4: "GBTN_ERR_TIMEOUT",
    5: "GBTN_ERR_NUMERIC",
    6: "GBTN_ERR_NOMEM",
}
HOST, DEVICE = 0, 1
KCLASS_TENSOR_CORE, KCLASS_SIMT_F32, KCLASS_SIMT_F64, KCLASS_GAUGE, KCLASS_SIMT_DF32 = 0, 1, 2, 3, 4
TC_POLICIES = {"auto": 0, "all": 1, "native": 2, "off": 3}
SCHED = {"sequential": 0, "parallel": 1, "colored": 2}
PRECISION = {"f64": 0, "f32": 1, "bf16": 2, "mixed": 3, "df32": 4}
REFINE = {"df32": 0, "f64": 1}
INIT = {"identity": 0, "ones": 1}


class LibraryNotBuilt(RuntimeError):
    pass


class GBTNError(RuntimeError):
    """Raised for a nonzero status; the reference raises ``error(...)`` at the
    same places (missing maxiter, bad arguments)."""

    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class InvalidArgument(GBTNError, ValueError):
    pass


class Unsupported(GBTNError, NotImplementedError):
    pass


class GraphDesc(C.Structure):
    _fields_ = [
        ("nv", C.c_int32),
        ("ne", C.c_int32),
        ("edge_u", C.POINTER(C.c_int32)),
        ("edge_v", C.POINTER(C.c_int32)),
        ("edge_dim", C.POINTER(C.c_int32)),
        ("site_dim", C.POINTER(C.c_int32)),
        ("leg_ptr", C.POINTER(C.c_int32)),
        ("leg_edge", C.POINTER(C.c_int32)),
        ("vertex_network", C.POINTER(C.c_int32)),
        ("n_networks", C.c_int32),
        ("separate_bra", C.c_int32),
        ("complex_values", C.c_int32),
    ]


class BPOpts(C.Structure):
    _fields_ = [
        ("schedule", C.c_int32),
        ("precision", C.c_int32),
        ("maxiter", C.c_int32),
        ("normalize", C.c_int32),
        ("tol", C.c_double),
        ("edge_sequence", C.POINTER(C.c_int32)),
        ("edge_sequence_len", C.c_int32),
        ("tol_bf16", C.c_double),
        ("tol_f32", C.c_double),
        ("maxiter_bf16", C.c_int32),
        ("maxiter_f32", C.c_int32),
        ("refine_f64", C.c_int32),
        ("refine", C.c_int32),
        ("confirm_f64", C.c_int32),
    ]


class QNDesc(C.Structure):
    _fields_ = [
        ("edge_sec_ptr", C.POINTER(C.c_int32)),
        ("sec_dim", C.POINTER(C.c_int32)),
        ("sec_charge", C.POINTER(C.c_int32)),
        ("site_sec_ptr", C.POINTER(C.c_int32)),
        ("site_sec_dim", C.POINTER(C.c_int32)),
        ("site_sec_charge", C.POINTER(C.c_int32)),
        ("flux", C.POINTER(C.c_int32)),
    ]


class GradOpts(C.Structure):
    _fields_ = [
        ("mode", C.c_int32),
        ("maxiter", C.c_int32),
        ("tol", C.c_double),
        ("unroll", C.c_int32),
        ("checkpoint", C.c_int32),
    ]


_P = C.c_void_p
_I = C.c_int
_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)

SIGNATURES = {
    "gbtn_abi_version": (_I, []),
    "gbtn_last_error": (C.c_char_p, [_P]),
    "gbtn_ctx_create": (_I, [_I, C.POINTER(_P)]),
    "gbtn_ctx_destroy": (_I, [_P]),
    "gbtn_ctx_set_stream": (_I, [_P, _P]),
    "gbtn_ctx_get_stream": (_P, [_P]),
    "gbtn_ctx_set_profiling": (_I, [_P, _I]),
    "gbtn_ctx_test_wait_timeout": (_I, [_P, _I]),
    "gbtn_ctx_kernel_time": (_I, [_P, _I, _D, C.POINTER(C.c_int64)]),
    "gbtn_plan_create": (_I, [_P, C.POINTER(GraphDesc), C.POINTER(_P)]),
    "gbtn_plan_destroy": (_I, [_P]),
    "gbtn_plan_sizes": (_I, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "gbtn_plan_set_tc_policy": (_I, [_P, C.c_int32]),
    "gbtn_plan_tc_split": (_I, [_P, _I32, _D]),
    "gbtn_plan_set_simt_tuning": (_I, [_P, C.c_int32]),
    "gbtn_plan_simt_teams": (_I, [_P, C.c_int32, _I32]),
    "gbtn_plan_set_graphs": (_I, [_P, C.c_int32]),
    "gbtn_set_factors": (_I, [_P, _P, _P, _I]),
    "gbtn_get_factors": (_I, [_P, _P, _I]),
    "gbtn_set_messages": (_I, [_P, _P, _I]),
    "gbtn_get_messages": (_I, [_P, _P, _I]),
    "gbtn_get_edge_diffs": (_I, [_P, _P, _I]),
    "gbtn_init_messages": (_I, [_P, _I]),
    "gbtn_bp_run": (_I, [_P, C.POINTER(BPOpts), _I32, _D]),
    "gbtn_plan_phase_sweeps": (_I, [_P, _I32]),
    "gbtn_plan_counters": (_I, [_P, C.POINTER(C.c_int64)]),
    "gbtn_updated_message": (_I, [_P, C.c_int32, _D]),
    "gbtn_vertex_rdms": (_I, [_P, _D]),
    "gbtn_expect1": (_I, [_P, _D, _I, _D]),
    "gbtn_edge_rdms": (_I, [_P, _I32, C.c_int32, _D]),
    "gbtn_expect2": (_I, [_P, _I32, C.c_int32, _D, _D]),
    "gbtn_vertex_scalars": (_I, [_P, _D]),
    "gbtn_edge_scalars": (_I, [_P, _D]),
    "gbtn_logscalar": (_I, [_P, _D, _D]),
    "gbtn_rescale_messages": (_I, [_P]),
    "gbtn_rescale_partitions": (_I, [_P]),
    "gbtn_su_create": (_I, [_P, C.POINTER(GraphDesc), C.c_int32, C.POINTER(_P)]),
    "gbtn_su_destroy": (_I, [_P]),
    "gbtn_su_edge_dims": (_I, [_P, _I32]),
    "gbtn_su_set_factors": (_I, [_P, _D]),
    "gbtn_su_get_factors": (_I, [_P, _D, C.c_int64]),
    "gbtn_su_apply": (_I, [_P, C.c_int32, _I32, _D, C.c_int32, _D, C.c_int32, C.c_double, C.c_int32, _D, _D]),
    "gbtn_su_set_edge_dims": (_I, [_P, _I32]),
    "gbtn_su_apply_vjp": (_I, [_P, C.c_int32, _I32, _D, C.c_int32, _D, C.c_int32, C.c_double, C.c_int32, _I32, _D,
                               _D, _D, _D]),
    "gbtn_su_apply_taped": (_I, [_P, C.c_int32, _I32, _D, C.c_int32, _D, C.c_int32, C.c_double, C.c_int32, _D, _D,
                                 C.POINTER(_P)]),
    "gbtn_su_tape_vjp": (_I, [_P, _P, _D, _D, _D, _D]),
    "gbtn_su_tape_destroy": (_I, [_P]),
    "gbtn_energy2": (_I, [_P, C.c_int32, _D, _D, _D]),
    "gbtn_energy2_grad": (_I, [_P, C.c_int32, _D, _D, C.POINTER(GradOpts), _D, _D, _I32, _D]),
    "gbtn_bp_vjp": (_I, [_P, _D, C.POINTER(GradOpts), _D, _I32, _D]),
    "gbtn_bp_sweep_static": (_I, [_I, C.POINTER(GraphDesc), _P, _P, _P, _P, _P]),
    "gbtn_logscalar_grad": (_I, [_P, C.POINTER(GradOpts), _D, _D, _I32, _D]),
    "gbtn_expect1_grad": (_I, [_P, _D, C.POINTER(GradOpts), _D, _D, _I32, _D]),
    "gbtn_qn_plan_create": (_I, [_P, C.POINTER(GraphDesc), C.POINTER(QNDesc), C.POINTER(_P)]),
    "gbtn_qn_plan_destroy": (_I, [_P]),
    "gbtn_qn_plan_sizes": (_I, [_P, _I32, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "gbtn_qn_blocks": (_I, [_P, _I32, C.POINTER(C.c_int64)]),
    "gbtn_qn_set_blocks": (_I, [_P, _P, _I]),
    "gbtn_qn_init_messages": (_I, [_P]),
    "gbtn_qn_set_messages": (_I, [_P, _P, _I]),
    "gbtn_qn_get_messages": (_I, [_P, _P, _I]),
    "gbtn_qn_bp_run": (_I, [_P, C.c_int32, C.c_double, _I32, _D]),
    "gbtn_qn_bp_run_sequential": (_I, [_P, _I32, C.c_int32, C.c_int32, C.c_double, _I32, _D]),
    "gbtn_qn_bp_run_ex": (_I, [_P, C.POINTER(BPOpts), _I32, _D]),
    "gbtn_qn_phase_sweeps": (_I, [_P, _I32]),
    "gbtn_qn_vertex_rdms": (_I, [_P, _D]),
    "gbtn_qn_logscalar": (_I, [_P, _D, _D]),
}


def declared_symbols(header: Path = INCLUDE / "gbtn.h"):
    """Function names declared in the C header (for the export check)."""
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbtn_[a-z0-9_]+)\s*\(", text)))


_lib = None


def load(path: Path | None = None):
    """Load libgbtn.so and attach signatures (cached)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise LibraryNotBuilt(f"{p} is missing: run gbtn.build.build() (nvcc, sm_103a) first")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(ctx, code):
    if code == GBTN_OK:
        return
    msg = load().gbtn_last_error(ctx).decode(errors="replace")
    if code == 1:
        raise InvalidArgument(code, msg)
    if code == 3:
        raise Unsupported(code, msg)
    raise GBTNError(code, msg)


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_D)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_I32)


class Context:
    """One CUDA device context of the library (gbtn_ctx_create)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        check(None, self.lib.gbtn_ctx_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    def set_stream(self, stream_ptr: int | None):
        check(self.handle, self.lib.gbtn_ctx_set_stream(self.handle, C.c_void_p(stream_ptr or 0)))

    def set_profiling(self, on: bool):
        check(self.handle, self.lib.gbtn_ctx_set_profiling(self.handle, 1 if on else 0))

    def kernel_time(self, kernel_class: int):
        """(total ms, launches) of one kernel class since the last read."""
        ms = C.c_double()
        n = C.c_int64()
        check(self.handle, self.lib.gbtn_ctx_kernel_time(self.handle, kernel_class, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    @property
    def stream(self) -> int:
        return self.lib.gbtn_ctx_get_stream(self.handle) or 0

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gbtn_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx
