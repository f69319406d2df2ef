"""ctypes bindings of librimu_gpu (include/rimu_gpu.h).

The library is the only compute path: if it cannot be loaded, or no CUDA device is present,
every call raises ``RimuError`` -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

RIMU_OK, RIMU_ERR_BADARG, RIMU_ERR_OOM, RIMU_ERR_OVERFLOW = 0, 1, 2, 3
RIMU_ERR_TIMEOUT, RIMU_ERR_CUDA, RIMU_ERR_STATE = 4, 5, 6
VAL_F64, VAL_I64 = 0, 1
MODEL_REAL1D, MODEL_REALSPACE, MODEL_MOM1D = 1, 2, 3
STYLE_INTEGER, STYLE_DETERMINISTIC, STYLE_DSS = 0, 1, 2
OP_TRANSITION, OP_HAMILTONIAN = 0, 1
ANN_HASH, ANN_SORT = 0, 1
MAX_COMPONENTS = 4          # RIMU_MAX_COMPONENTS

# Names of the C entry points declared in include/rimu_gpu.h.
EXPORTS = [
    "rimu_version", "rimu_last_error", "rimu_ctx_create", "rimu_ctx_destroy",
    "rimu_ctx_synchronize", "rimu_model_create", "rimu_model_destroy", "rimu_model_diagonal",
    "rimu_model_num_offdiagonals", "rimu_model_offdiagonals", "rimu_model_num_offdiagonals_w",
    "rimu_model_offdiagonals_w", "rimu_vec_create", "rimu_vec_create_kw", "rimu_vec_key_words",
    "rimu_vec_destroy", "rimu_vec_upload", "rimu_vec_download", "rimu_vec_length",
    "rimu_vec_walkernumber_and_length", "rimu_vec_lookup", "rimu_vec_copy", "rimu_vec_empty",
    "rimu_wm_create", "rimu_wm_destroy", "rimu_wm_set_projector", "rimu_wm_set_timing",
    "rimu_wm_set_launch_shape", "rimu_wm_set_annihilation", "rimu_wm_set_projector_w",
    "rimu_vec_scale", "rimu_vec_add",
    "rimu_wm_timing", "rimu_apply_operator",
    "rimu_basis_dimension", "rimu_basis_keys", "rimu_hv_basis", "rimu_hv_basis_adjoint",
    "rimu_hv_basis_adjoint_noalloc",
    "rimu_batch_create", "rimu_batch_destroy", "rimu_batch_set_replica", "rimu_batch_set_projector",
    "rimu_batch_set_launch_shape", "rimu_batch_run", "rimu_batch_download", "rimu_batch_info",
    "rimu_batch_set_annihilation", "rimu_batch_annihilation",
    "rimu_vec_dot", "rimu_vec_convert",
]


class RimuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[rimu status {code}] {msg}")
        self.code = code


class ModelDesc(C.Structure):
    _fields_ = [("kind", C.c_int), ("fermion", C.c_int), ("n_particles", C.c_int),
                ("n_modes", C.c_int), ("u", C.c_double), ("t", C.c_double), ("ndim", C.c_int),
                ("dims", C.c_int * 3), ("periodic", C.c_int * 3),
                ("potential", C.POINTER(C.c_double)), ("dispersion", C.POINTER(C.c_double)),
                ("n_components", C.c_int), ("comp_fermion", C.c_int * MAX_COMPONENTS),
                ("comp_particles", C.c_int * MAX_COMPONENTS),
                ("comp_t", C.c_double * MAX_COMPONENTS),
                ("comp_u", C.c_double * (MAX_COMPONENTS * (MAX_COMPONENTS + 1) // 2))]


class StepParams(C.Structure):
    _fields_ = [("style", C.c_int), ("op", C.c_int), ("dt", C.c_double), ("shift", C.c_double),
                ("boost", C.c_double), ("proj_threshold", C.c_double),
                ("compression", C.c_double), ("rel_spawning_threshold", C.c_double),
                ("abs_spawning_threshold", C.c_double), ("seed", C.c_uint64),
                ("step", C.c_uint64), ("replica", C.c_uint32), ("initiator", C.c_int),
                ("initiator_threshold", C.c_double)]


class StepStats(C.Structure):
    _fields_ = [("norm", C.c_double), ("len", C.c_int64), ("len_before", C.c_int64),
                ("exact_steps", C.c_int64), ("inexact_steps", C.c_int64),
                ("spawn_attempts", C.c_int64), ("spawns", C.c_double), ("clones", C.c_int64),
                ("deaths", C.c_int64), ("zombies", C.c_int64), ("vproj", C.c_double),
                ("hproj", C.c_double), ("spawn_records", C.c_int64), ("retries", C.c_int32),
                ("nb_bits", C.c_int32)]


class BatchParams(C.Structure):
    _fields_ = [("style", C.c_int), ("dt", C.c_double), ("boost", C.c_double),
                ("proj_threshold", C.c_double), ("compression", C.c_double),
                ("rel_spawning_threshold", C.c_double), ("abs_spawning_threshold", C.c_double),
                ("seed", C.c_uint64), ("shift_update", C.c_int), ("zeta", C.c_double),
                ("xi", C.c_double), ("segment_steps", C.c_int), ("use_graph", C.c_int),
                ("autotune", C.c_int)]


class BatchStats(C.Structure):
    _fields_ = [("shift", C.c_double), ("norm", C.c_double), ("vproj", C.c_double),
                ("hproj", C.c_double), ("spawns", C.c_double), ("len", C.c_int64),
                ("len_before", C.c_int64), ("exact_steps", C.c_int64),
                ("inexact_steps", C.c_int64), ("spawn_attempts", C.c_int64),
                ("spawn_records", C.c_int64), ("clones", C.c_int64), ("deaths", C.c_int64),
                ("zombies", C.c_int64)]


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load librimu_gpu.so (building it with nvcc when it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build_if_missing else _build.LIB
    if not os.path.exists(path):
        raise RimuError(RIMU_ERR_STATE, f"librimu_gpu not built: {path} missing")
    lib = C.CDLL(path)
    P = C.POINTER
    vp, u64p, f64p, i64p = C.c_void_p, P(C.c_uint64), P(C.c_double), P(C.c_int64)
    sig = {
        "rimu_version": ([], C.c_int),
        "rimu_last_error": ([C.c_char_p, C.c_size_t], C.c_int),
        "rimu_ctx_create": ([C.c_int, vp, P(vp)], C.c_int),
        "rimu_ctx_destroy": ([vp], C.c_int),
        "rimu_ctx_synchronize": ([vp], C.c_int),
        "rimu_model_create": ([vp, P(ModelDesc), P(vp)], C.c_int),
        "rimu_model_destroy": ([vp], C.c_int),
        "rimu_model_diagonal": ([vp, u64p, C.c_int64, f64p], C.c_int),
        "rimu_model_num_offdiagonals": ([vp, C.c_uint64, P(C.c_int)], C.c_int),
        "rimu_model_offdiagonals": ([vp, C.c_uint64, u64p, f64p, C.c_int, P(C.c_int)], C.c_int),
        "rimu_vec_create": ([vp, C.c_int, C.c_int64, P(vp)], C.c_int),
        "rimu_vec_create_kw": ([vp, C.c_int, C.c_int, C.c_int64, P(vp)], C.c_int),
        "rimu_vec_key_words": ([vp, P(C.c_int)], C.c_int),
        "rimu_model_num_offdiagonals_w": ([vp, u64p, P(C.c_int)], C.c_int),
        "rimu_model_offdiagonals_w": ([vp, u64p, u64p, f64p, C.c_int, P(C.c_int)], C.c_int),
        "rimu_vec_destroy": ([vp], C.c_int),
        "rimu_vec_upload": ([vp, u64p, vp, C.c_int64], C.c_int),
        "rimu_vec_download": ([vp, u64p, vp, C.c_int64, i64p], C.c_int),
        "rimu_vec_length": ([vp, i64p], C.c_int),
        "rimu_vec_walkernumber_and_length": ([vp, f64p, i64p], C.c_int),
        "rimu_vec_lookup": ([vp, u64p, C.c_int64, vp], C.c_int),
        "rimu_vec_copy": ([vp, vp], C.c_int),
        "rimu_vec_empty": ([vp], C.c_int),
        "rimu_wm_create": ([vp, P(vp)], C.c_int),
        "rimu_wm_destroy": ([vp], C.c_int),
        "rimu_wm_set_projector": ([vp, u64p, f64p, f64p, C.c_int], C.c_int),
        "rimu_wm_set_projector_w": ([vp, u64p, f64p, f64p, C.c_int], C.c_int),
        "rimu_vec_scale": ([vp, C.c_double], C.c_int),
        "rimu_vec_add": ([vp, vp, C.c_double, C.c_double], C.c_int),
        "rimu_wm_set_timing": ([vp, C.c_int], C.c_int),
        "rimu_wm_set_launch_shape": ([vp, C.c_int, C.c_int], C.c_int),
        "rimu_wm_set_annihilation": ([vp, C.c_int], C.c_int),
        "rimu_wm_timing": ([vp, f64p], C.c_int),
        "rimu_apply_operator": ([vp, vp, vp, vp, P(StepParams), P(StepStats)], C.c_int),
        "rimu_basis_dimension": ([vp, i64p], C.c_int),
        "rimu_basis_keys": ([vp, C.c_int64, C.c_int64, u64p], C.c_int),
        "rimu_hv_basis": ([vp, vp, vp, C.c_int64], C.c_int),
        "rimu_hv_basis_adjoint": ([vp, vp, vp, vp, f64p, f64p, C.c_int64], C.c_int),
        "rimu_hv_basis_adjoint_noalloc": ([P(ModelDesc), vp, vp, vp, f64p, f64p, C.c_int64, vp],
                                          C.c_int),
        "rimu_batch_create": ([vp, C.c_int, C.c_int, P(vp)], C.c_int),
        "rimu_batch_destroy": ([vp], C.c_int),
        "rimu_batch_set_replica": ([vp, C.c_int, vp, u64p, vp, C.c_int64, C.c_double, C.c_double],
                                   C.c_int),
        "rimu_batch_set_projector": ([vp, C.c_int, u64p, f64p, f64p, C.c_int], C.c_int),
        "rimu_batch_set_launch_shape": ([vp, C.c_int, C.c_int], C.c_int),
        "rimu_batch_set_annihilation": ([vp, C.c_int], C.c_int),
        "rimu_batch_annihilation": ([vp, C.POINTER(C.c_int)], C.c_int),
        "rimu_batch_run": ([vp, P(BatchParams), C.c_uint64, C.c_int, vp], C.c_int),
        "rimu_batch_download": ([vp, C.c_int, u64p, vp, C.c_int64, i64p], C.c_int),
        "rimu_batch_info": ([vp, f64p], C.c_int),
        "rimu_vec_dot": ([vp, vp, f64p], C.c_int),
        "rimu_vec_convert": ([vp, vp, C.c_int], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    load().rimu_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(rc: int):
    if rc != RIMU_OK:
        raise RimuError(rc, last_error())


# ------------------------------------------------------------------------------------------
# Default context (one per process and device, on torch's current stream when available)
# ------------------------------------------------------------------------------------------
class Context:
    def __init__(self, device: int = 0, stream: int | None = None):
        lib = load()
        h = C.c_void_p()
        check(lib.rimu_ctx_create(device, C.c_void_p(stream) if stream else None, C.byref(h)))
        self.stream = stream or 0
        self.handle = h
        self.device = device
        self._lib = lib

    def synchronize(self):
        check(self._lib.rimu_ctx_synchronize(self.handle))

    def __del__(self):
        try:
            if self.handle:
                self._lib.rimu_ctx_destroy(self.handle)
        except Exception:
            pass


_ctx: Context | None = None


def default_context() -> Context:
    """The process-wide context on CUDA device 0, bound to torch's current stream."""
    global _ctx
    if _ctx is None:
        stream = None
        try:
            import torch
            if torch.cuda.is_available():
                stream = torch.cuda.current_stream(0).cuda_stream
        except ImportError:
            pass
        _ctx = Context(0, stream)
    return _ctx
