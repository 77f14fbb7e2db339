"""ctypes binding of libphylo_gpu.so (the C ABI declared in include/phylo_gpu.h).

This is the only route from Python to the GPU kernels.  There is no CPU
fallback: if the shared object is missing or no sm_100-family device is
present, calls raise ``NativeError``.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libphylo_gpu.so"

PGPU_OK = 0
STATUS_NAMES = {
    0: "PGPU_OK", 1: "PGPU_ERR_ARG", 2: "PGPU_ERR_CUDA", 3: "PGPU_ERR_OOM",
    4: "PGPU_ERR_NAN", 5: "PGPU_ERR_NONREVERSIBLE", 6: "PGPU_ERR_EIGEN",
    7: "PGPU_ERR_OVERFLOW", 8: "PGPU_ERR_TIMEOUT", 9: "PGPU_ERR_UNSUPPORTED",
    10: "PGPU_ERR_LIMIT",
}


class NativeError(RuntimeError):
    """A C-ABI call failed (status != PGPU_OK), or the library is missing.

    Mirrors the reference's ``failwith`` on LAPACK errors (lib/mlmodel.c:110-120):
    the message is the library's own.
    """

    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class PgpuTree(C.Structure):
    _fields_ = [
        ("n_tips", C.c_int32),
        ("left", C.POINTER(C.c_int32)),
        ("right", C.POINTER(C.c_int32)),
        ("brlen", C.POINTER(C.c_double)),
    ]


class PgpuModel(C.Structure):
    _fields_ = [
        ("n_states", C.c_int32),
        ("n_rates", C.c_int32),
        ("Q", C.POINTER(C.c_double)),
        ("pi", C.POINTER(C.c_double)),
        ("rates", C.POINTER(C.c_double)),
        ("probs", C.POINTER(C.c_double)),
    ]


class PgpuTipCodes(C.Structure):
    _fields_ = [
        ("n_codes", C.c_int32),
        ("table", C.POINTER(C.c_double)),
    ]


class PgpuBatchOptions(C.Structure):
    _fields_ = [("rate_pairs", C.c_int), ("order", C.c_int)]


class PgpuVariant(C.Structure):
    _fields_ = [
        ("tree", PgpuTree),
        ("model", PgpuModel),
        ("codes", PgpuTipCodes),
        ("tip_codes", C.c_void_p),
        ("weights", C.c_void_p),
        ("n_pat", C.c_size_t),
        ("ld_pat", C.c_size_t),
    ]


_P = C.c_void_p
_SZ = C.c_size_t
_I = C.c_int
_U64P = C.POINTER(C.c_uint64)
_DP = C.POINTER(C.c_double)

# name -> (restype, argtypes); the complete list of exported entry points
SIGNATURES: dict[str, tuple] = {
    "pgpu_create": (_I, [C.POINTER(_P), _I]),
    "pgpu_destroy": (None, [_P]),
    "pgpu_last_error": (C.c_char_p, [_P]),
    "pgpu_set_stream": (_I, [_P, _P]),
    "pgpu_synchronize": (_I, [_P]),
    "pgpu_kernel_launches": (C.c_uint64, [_P]),
    "pgpu_get_stream": (_P, [_P]),
    "pgpu_version": (_I, []),
    "pgpu_tree_schedule": (_I, [_P, C.POINTER(PgpuTree), _P, C.POINTER(C.c_int32)]),
    "pgpu_fitch_median2": (_I, [_P, _P, _P, _P, _SZ, _I, _U64P]),
    "pgpu_fitch_median2_weighted": (_I, [_P, _P, _P, _P, _P, _SZ, _I, _U64P]),
    "pgpu_fitch_distance": (_I, [_P, _P, _P, _SZ, _I, _U64P]),
    "pgpu_set_fitch_tile_words": (_I, [_P, _I]),
    "pgpu_get_fitch_tile_words": (_I, [_P]),
    "pgpu_nonadditive_median2": (_I, [_P, _P, _P, _P, _P, _SZ, _DP]),
    "pgpu_fitch_tree": (_I, [_P, C.POINTER(PgpuTree), _P, _P, _SZ, _I, _P, _P, _U64P]),
    "pgpu_fitch_tree_dev": (_I, [_P, C.POINTER(PgpuTree), _P, _SZ, _P, _SZ, _I, _P, _P, _P]),
    "pgpu_fitch_tree_noalloc": (_I, [C.POINTER(PgpuTree), _P, _SZ, _P, _SZ, _I, _P, _P, _P, _P]),
    "pgpu_tcm_tables": (_I, [_P, _P, _I, _I, _I, _P, _P, _P]),
    "pgpu_tcm_tree": (_I, [_P, C.POINTER(PgpuTree), _P, _P, _SZ, _P, _P, _P, _P]),
    "pgpu_tcm_tree_dev": (_I, [_P, C.POINTER(PgpuTree), _P, _SZ, _P, _SZ, _P, _P, _P, _P]),
    "pgpu_tcm_tree_wide": (_I, [_P, C.POINTER(PgpuTree), _P, _P, _SZ, _I, _P, _I, _I, _I, _P, _P, _P]),
    "pgpu_tcm_median": (_I, [_P, _I, _I, _I, C.c_uint32, C.c_uint32, C.POINTER(C.c_int64),
                             C.POINTER(C.c_uint32)]),
    "pgpu_tcm_tree_wide_dev": (_I, [_P, C.POINTER(PgpuTree), _P, _SZ, _P, _SZ, _I, _P, _I, _I, _I,
                                    _P, _P, _P]),
    "pgpu_model_diagonalize": (_I, [_P, _P, _P, _I, _P, _P, _P]),
    "pgpu_model_compose": (_I, [_P, _P, _P, _P, _I, _P, _SZ, _P]),
    "pgpu_diagonalize_gtr": (_I, [_P, _P, _P, _P, _I]),
    "pgpu_diagonalize_sym": (_I, [_P, _P, _P, _I]),
    "pgpu_compose_gtr": (_I, [_P, _P, _P, _P, _I, C.c_double, _P]),
    "pgpu_compose_sym": (_I, [_P, _P, _P, _I, C.c_double, _P]),
    "pgpu_prune_lnl": (_I, [_P, C.POINTER(PgpuTree), C.POINTER(PgpuModel),
                            C.POINTER(PgpuTipCodes), _P, _P, _SZ, _I, _DP, _P]),
    "pgpu_prune_lnl_dev": (_I, [_P, C.POINTER(PgpuTree), C.POINTER(PgpuModel),
                                C.POINTER(PgpuTipCodes), _P, _SZ, _P, _SZ, _I, _P, _P]),
    "pgpu_prune_lnl_models": (_I, [_P, C.POINTER(PgpuTree), C.POINTER(PgpuModel), _I,
                                   C.POINTER(PgpuTipCodes), _P, _P, _SZ, _I, _P]),
    "pgpu_prune_lnl_models_dev": (_I, [_P, C.POINTER(PgpuTree), C.POINTER(PgpuModel), _I,
                                       C.POINTER(PgpuTipCodes), _P, _SZ, _P, _SZ, _I, _P]),
    "pgpu_lk_create": (_I, [_P, C.POINTER(PgpuModel), C.POINTER(PgpuTipCodes), _SZ, _P, _I,
                            C.POINTER(_P)]),
    "pgpu_lk_destroy": (None, [_P]),
    "pgpu_clv_leaf": (_I, [_P, _P, _P, C.POINTER(_P)]),
    "pgpu_clv_set_brlen": (_I, [_P, C.c_double]),
    "pgpu_clv_get_brlen": (_I, [_P, _DP]),
    "pgpu_clv_median1": (_I, [_P, _P, _P, C.POINTER(_P)]),
    "pgpu_clv_median2": (_I, [_P, _P, _P, _P, C.POINTER(_P)]),
    "pgpu_clv_median3": (_I, [_P, _P, _P, _P, _P, C.POINTER(_P)]),
    "pgpu_clv_cost": (_I, [_P, _DP]),
    "pgpu_clv_costs": (_I, [_P, _P, _SZ, _P]),
    "pgpu_clv_root_cost": (_I, [_P, _DP, _P]),
    "pgpu_clv_destroy": (None, [_P]),
    "pgpu_batch_create": (_I, [_P, C.POINTER(PgpuVariant), _I, C.POINTER(_P)]),
    "pgpu_batch_create_opts": (_I, [_P, C.POINTER(PgpuVariant), _I, C.POINTER(PgpuBatchOptions),
                                    C.POINTER(_P)]),
    "pgpu_batch_destroy": (None, [_P]),
    "pgpu_batch_run": (_I, [_P, _P, _P, _P]),
    "pgpu_batch_run_fp64": (_I, [_P, _P, _SZ, _P]),
    "pgpu_batch_work_items": (C.c_longlong, [_P]),
    "pgpu_batch_patterns": (C.c_longlong, [_P]),
    "pgpu_spr_create": (_I, [_P, C.POINTER(PgpuModel), C.POINTER(PgpuTipCodes), C.c_int32, _P, _SZ,
                             _P, _SZ, _I, C.POINTER(_P)]),
    "pgpu_spr_destroy": (None, [_P]),
    "pgpu_spr_set_tree": (_I, [_P, C.POINTER(PgpuTree)]),
    "pgpu_spr_get_tree": (_I, [_P, _P, _P, _P]),
    "pgpu_spr_lnl": (_I, [_P, _DP, _P]),
    "pgpu_spr_set_join_distance": (_I, [_P, _I]),
    "pgpu_spr_set_tbr_distance": (_I, [_P, _I]),
    "pgpu_spr_set_tbr_limits": (_I, [_P, _I, _I]),
    "pgpu_spr_set_tbr_budget": (_I, [_P, _SZ]),
    "pgpu_spr_tbr_n_moves": (_I, [_P, C.POINTER(_SZ)]),
    "pgpu_spr_tbr_moves": (_I, [_P, _P, _P, _P, _P, _P, _P, _SZ]),
    "pgpu_spr_tbr_scan": (_I, [_P, _P]),
    "pgpu_spr_tbr_apply": (_I, [_P, C.c_int64]),
    "pgpu_spr_n_moves": (_I, [_P, C.POINTER(_SZ)]),
    "pgpu_spr_moves": (_I, [_P, _P, _P, _P, _P, _SZ]),
    "pgpu_spr_scan": (_I, [_P, _P]),
    "pgpu_spr_score": (_I, [_P, _P, _SZ, _P]),
    "pgpu_spr_fitch": (_I, [_P, _P, _U64P]),
    "pgpu_spr_features": (_I, [_P, _P]),
    "pgpu_spr_apply": (_I, [_P, C.c_int64]),
    "pgpu_spr_optimize": (_I, [_P, _I, C.c_double, _DP]),
    "pgpu_spr_lengths": (_I, [_P, _P, _P, _P]),
    "pgpu_mlp_n_params": (C.c_longlong, []),
    "pgpu_mlp_create": (_I, [_P, C.c_uint64, _I, C.POINTER(_P)]),
    "pgpu_mlp_destroy": (None, [_P]),
    "pgpu_mlp_get_params": (_I, [_P, _P]),
    "pgpu_mlp_set_params": (_I, [_P, _P]),
    "pgpu_mlp_get_norm": (_I, [_P, _P, _P]),
    "pgpu_mlp_fit_norm": (_I, [_P, _P, _SZ]),
    "pgpu_mlp_forward": (_I, [_P, _P, _SZ, _P]),
    "pgpu_mlp_grads": (_I, [_P, _P, _P, _P, _SZ, _P, C.POINTER(C.c_float)]),
    "pgpu_mlp_train_step": (_I, [_P, _P, _P, _P, _SZ, C.c_float, C.c_float,
                                 C.POINTER(C.c_float)]),
    "pgpu_parsimony_stepwise": (_I, [C.c_int32, _P, _SZ, _SZ, _P, _I, _P, C.c_uint64, C.c_double,
                                     _P, _P, _P, _U64P]),
}

_lib = None
_lock = threading.RLock()   # default_context() holds it while load() takes it


def load() -> C.CDLL:
    """Loads libphylo_gpu.so and declares every signature; raises if absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not LIB_PATH.exists():
            raise NativeError(9, f"{LIB_PATH} is missing; build it with phylocaml_gb300.build.build()")
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def ptr(a) -> int | None:
    """Address of a numpy array's data, a torch tensor's data, or None."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if isinstance(a, int):
        return a
    raise TypeError(f"cannot take the address of {type(a)}")


def make_tree(left: np.ndarray, right: np.ndarray, brlen: np.ndarray | None = None):
    """Builds a PgpuTree; returns (struct, keepalive) -- keep both alive."""
    left = np.ascontiguousarray(left, dtype=np.int32)
    right = np.ascontiguousarray(right, dtype=np.int32)
    keep = [left, right]
    t = PgpuTree()
    t.n_tips = len(left) + 1
    t.left = left.ctypes.data_as(C.POINTER(C.c_int32))
    t.right = right.ctypes.data_as(C.POINTER(C.c_int32))
    if brlen is not None:
        brlen = np.ascontiguousarray(brlen, dtype=np.float64)
        keep.append(brlen)
        t.brlen = brlen.ctypes.data_as(C.POINTER(C.c_double))
    return t, keep


class Context:
    """Owns one pgpu_ctx (device memory and a stream) on one GPU."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = _P()
        st = self.lib.pgpu_create(C.byref(h), device)
        if st != PGPU_OK:
            raise NativeError(st, f"pgpu_create(device={device}) failed "
                                  "(needs an sm_100-family GPU and the CUDA runtime)")
        self.h = h
        self.device = device

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.pgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def check(self, st: int, what: str) -> None:
        if st != PGPU_OK:
            msg = self.lib.pgpu_last_error(self.h)
            raise NativeError(st, f"{what}: {msg.decode() if msg else ''}")

    def call(self, name: str, *args) -> None:
        self.check(getattr(self.lib, name)(self.h, *args), name)

    @property
    def launches(self) -> int:
        return int(self.lib.pgpu_kernel_launches(self.h))

    def set_stream(self, stream_handle: int | None) -> None:
        self.call("pgpu_set_stream", stream_handle)

    def synchronize(self) -> None:
        self.call("pgpu_synchronize")

    # The context's stream is a non-blocking CUDA stream: it does not wait
    # for PyTorch's current stream, nor PyTorch for it.  Wrappers that hand
    # tensors across call these around their asynchronous library calls.
    def _ext(self):
        import torch
        h = self.lib.pgpu_get_stream(self.h)
        if getattr(self, "_ext_handle", None) != h:
            self._ext_stream = torch.cuda.ExternalStream(h, device=torch.device("cuda", self.device))
            self._ext_handle = h
        return self._ext_stream

    def after_torch(self) -> None:
        """Library work issued from now on waits for PyTorch's queued work."""
        import torch
        self._ext().wait_stream(torch.cuda.current_stream(torch.device("cuda", self.device)))

    def before_torch(self) -> None:
        """PyTorch work issued from now on waits for the library's queued work."""
        import torch
        torch.cuda.current_stream(torch.device("cuda", self.device)).wait_stream(self._ext())


_default: Context | None = None


def default_context() -> Context:
    """A process-wide context on device 0, created on first use."""
    global _default
    with _lock:
        if _default is None:
            _default = Context(0)
        return _default


def tree_schedule(left: np.ndarray, right: np.ndarray):
    """Host-only schedule query: (ops [n_int, 3] int32, max stack depth)."""
    lib = load()
    t, keep = make_tree(left, right)
    ops = np.empty((len(keep[0]), 3), dtype=np.int32)
    depth = C.c_int32(0)
    st = lib.pgpu_tree_schedule(None, C.byref(t), ops.ctypes.data, C.byref(depth))
    if st != PGPU_OK:
        raise NativeError(st, "pgpu_tree_schedule: invalid tree")
    return ops, int(depth.value)
