"""ctypes binding of libpqgb300.so (the C ABI declared in include/pqgb300.h).

The library is required: importing the product API without it raises, there
is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PQ_OK = 0
PQ_ERR_INVALID = -1
PQ_ERR_NOT_FOUND = -2
PQ_ERR_OOM = -3
PQ_ERR_CUDA = -4
PQ_ERR_DEVICE = -5
PQ_ERR_UNSUPPORTED = -6

PQ_C64 = 1
PQ_C128 = 2

PREC_C128 = 0
PREC_C64 = 1
PREC_3XTF32 = 2
PREC_3XBF16 = 3
PREC_6XTF32 = 4
PREC_OZAKI = 5
PREC_OZAKI4 = 6

PQ_MAX_RANK = 56

_ERRNAMES = {
    PQ_ERR_INVALID: "PQ_ERR_INVALID",
    PQ_ERR_NOT_FOUND: "PQ_ERR_NOT_FOUND",
    PQ_ERR_OOM: "PQ_ERR_OOM",
    PQ_ERR_CUDA: "PQ_ERR_CUDA",
    PQ_ERR_DEVICE: "PQ_ERR_DEVICE",
    PQ_ERR_UNSUPPORTED: "PQ_ERR_UNSUPPORTED",
}


class PQError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{_ERRNAMES.get(code, code)}: {msg}")
        self.code = code


LIB_PATH = Path(os.environ.get("PQGB300_LIB", Path(__file__).resolve().parent / "lib" / "libpqgb300.so"))

_lib = None

i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
f64p = C.POINTER(C.c_double)
f32p = C.POINTER(C.c_float)
vp = C.c_void_p

# (name, restype, argtypes) for every exported function
SIGNATURES = [
    ("pq_ctx_create", C.c_int, [C.c_int, C.c_int, C.POINTER(vp)]),
    ("pq_ctx_destroy", C.c_int, [vp]),
    ("pq_last_error", C.c_char_p, [vp]),
    ("pq_ctx_precision", C.c_int, [vp]),
    ("pq_ctx_sync", C.c_int, [vp]),
    ("pq_ctx_set_mem_cap", C.c_int, [vp, C.c_int64]),
    ("pq_ctx_mem_in_use", C.c_int, [vp, i64p]),
    ("pq_ctx_launch_count", C.c_int, [vp, i64p]),
    ("pq_ctx_set_small_elems", C.c_int, [vp, C.c_int64]),
    ("pq_ctx_stream", C.c_int, [vp, C.POINTER(vp)]),
    ("pq_save_tensor_data", C.c_int, [vp, C.c_int64, C.c_int, i64p, vp, C.c_int]),
    ("pq_save_tensors", C.c_int, [vp, C.c_int, i64p, i32p, i64p, C.POINTER(C.c_void_p), i32p]),
    ("pq_load_tensor_data", C.c_int, [vp, C.c_int64, vp, C.c_int64, C.c_int]),
    ("pq_tensor_shape", C.c_int, [vp, C.c_int64, C.POINTER(C.c_int), i64p]),
    ("pq_has_tensor", C.c_int, [vp, C.c_int64]),
    ("pq_delete_tensor", C.c_int, [vp, C.c_int64]),
    ("pq_save_output", C.c_int, [vp, C.c_int64, C.c_int64]),
    ("pq_contract_tensors", C.c_int, [vp, C.c_int64, i32p, C.c_int, C.c_int64, i32p, C.c_int, C.c_int64]),
    ("pq_permute_tensor", C.c_int, [vp, C.c_int64, i32p, C.c_int]),
    ("pq_reshape_tensor", C.c_int, [vp, C.c_int64, C.c_int, i32p, i32p]),
    ("pq_view_tensor", C.c_int, [vp, C.c_int64, C.c_int64, C.c_int, C.c_int64, C.c_int64]),
    ("pq_tensor_norm2", C.c_int, [vp, C.c_int64, C.POINTER(C.c_double)]),
    ("pq_decompose_tensor", C.c_int, [vp, C.c_int64, C.c_int, i32p, C.c_int, i32p, C.c_double, C.c_int, C.c_int64,
                                      C.c_int64, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("pq_gather_elements", C.c_int, [vp, C.c_int64, i64p, C.c_int64, vp, C.c_int]),
    ("pq_gather_elements_noalloc", C.c_int, [vp, C.c_int64, i64p, C.c_int64, vp, C.c_int]),
    ("pq_plan_create", C.c_int, [vp, C.c_int, i32p, i32p, C.c_int, i64p, C.c_int, i32p, C.c_int, i32p,
                                 C.POINTER(vp)]),
    ("pq_plan_destroy", C.c_int, [vp]),
    ("pq_plan_info", C.c_int, [vp, f64p, i64p, i64p, i64p]),
    ("pq_plan_execute", C.c_int, [vp, i64p, C.c_int64]),
    ("pq_plan_capture", C.c_int, [vp, i64p, C.c_int64]),
    ("pq_plan_profile", C.c_int, [vp, i64p, C.c_int64, f32p]),
    ("pq_plan_step_features", C.c_int, [vp, f64p]),
    ("pq_plan_run_sliced", C.c_int, [vp, i64p, C.c_int, i32p, C.c_int64, C.c_int64, C.c_int, C.c_int]),
    ("pq_sliced_result", C.c_int, [vp, f64p, C.c_int64]),
    ("pq_plan_profile_sliced", C.c_int, [vp, i64p, C.c_int, i32p, C.c_int, f32p, i32p, f64p]),
    ("pq_plan_greedy", C.c_int, [C.c_int, i32p, i32p, C.c_int, i64p, C.c_int, i32p, C.c_double, C.c_double,
                                 C.c_int, C.c_uint64, i32p, f64p, i64p]),
    ("pq_plan_greedy_many", C.c_int, [C.c_int, i32p, i32p, C.c_int, i64p, C.c_int, i32p, C.c_double,
                                      C.c_double, C.c_int, C.c_uint64, C.c_int, i32p, f64p, i64p]),
    ("pq_plan_cost", C.c_int, [C.c_int, i32p, i32p, C.c_int, i64p, C.c_int, i32p, C.c_int, i32p, f64p, f64p]),
    ("pq_plan_choose_slices", C.c_int, [C.c_int, i32p, i32p, C.c_int, i64p, C.c_int, i32p, C.c_int, i32p,
                                        C.c_int, C.c_double, i32p, C.POINTER(C.c_int)]),
    ("pq_measure_pairs", C.c_int, [vp, C.c_int, i32p, i32p, i32p, i64p, C.c_int, f32p, f64p]),
    ("pq_mlp_create", C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_uint64, C.POINTER(vp)]),
    ("pq_mlp_destroy", C.c_int, [vp]),
    ("pq_mlp_num_params", C.c_int, [vp, i64p]),
    ("pq_mlp_get_params", C.c_int, [vp, f32p, C.c_int64]),
    ("pq_mlp_set_params", C.c_int, [vp, f32p, C.c_int64]),
    ("pq_mlp_gradients", C.c_int, [vp, f32p, f32p, C.c_int64, f32p, f32p]),
    ("pq_mlp_train", C.c_int, [vp, f32p, f32p, C.c_int64, C.c_int, C.c_int, C.c_float, C.c_uint64, f32p]),
    ("pq_mlp_predict", C.c_int, [vp, f32p, C.c_int64, f32p, C.c_int]),
    ("pq_selftest_wait_expiry", C.c_int, [vp, C.c_uint32, C.POINTER(C.c_int)]),
    ("pq_ctx_set_tuning", C.c_int, [vp, C.c_int, C.POINTER(C.c_uint64), i32p]),
    ("pq_ctx_tuning_size", C.c_int, [vp, C.POINTER(C.c_int)]),
    ("pq_device_name", C.c_int, [C.c_int, C.c_char_p, C.c_int]),
    ("pq_svbatch_create", C.c_int, [vp, C.c_int, i32p, i32p, i32p, i32p, f64p, i32p, i64p, C.c_int64,
                                    C.POINTER(vp)]),
    ("pq_svbatch_execute", C.c_int, [vp, f64p]),
    ("pq_svbatch_info", C.c_int, [vp, i64p, i64p, i64p]),
    ("pq_svbatch_destroy", C.c_int, [vp]),
    ("pq_plan_cost_batch", C.c_int, [vp, C.c_int, i32p, i32p, C.c_int, i64p, C.c_int, C.c_int, i32p, C.c_int, i32p,
                                     f64p, f64p]),
    ("pq_pair_tuning", C.c_int, [vp, C.c_int, C.c_int, i32p, i64p, C.POINTER(C.c_uint64), C.c_int, i32p,
                                 C.POINTER(C.c_int)]),
]

# exported by the library but optional for older builds
OPTIONAL = set()


def lib():
    """Load the shared library (once); raise if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"libpqgb300.so not found at {LIB_PATH}: build it first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    L = C.CDLL(str(LIB_PATH))
    for name, res, args in SIGNATURES:
        if not hasattr(L, name):
            if name in OPTIONAL:
                continue
            raise ImportError(f"libpqgb300.so does not export {name}")
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def arr(ctype, values):
    values = list(values)
    return (ctype * max(1, len(values)))(*values)


def check(code, ctx=None, what=""):
    if code == PQ_OK:
        return
    msg = ""
    if ctx is not None:
        try:
            msg = lib().pq_last_error(ctx).decode()
        except Exception:  # pragma: no cover
            msg = ""
    raise PQError(code, f"{what}: {msg}" if what else msg)
