"""ctypes binding of libbsg.so (the C ABI in include/bsg.h).

The shared library is built in-tree by ``bosonsupremacy_gb300.build``.  There
is no fallback: if the library or a CUDA device is missing, every entry point
raises ``BSGError``.  Tensors are torch CUDA tensors used as plain device
buffers (``data_ptr()``); the library never sees torch types.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbsg.so")

PREC_FP64, PREC_SPLIT, PREC_FP32, PREC_SLICED = 0, 1, 2, 3
PRECISIONS = {"fp64": PREC_FP64, "split": PREC_SPLIT, "fp32": PREC_FP32, "sliced": PREC_SLICED}
SITE_FIRST, SITE_MIDDLE, SITE_LAST = 0, 1, 2
K_DP, K_WILLIAMSON, K_THERMAL, K_SIGMA, K_PREP, K_CONTRACT, K_HOST_PLAN, K_HOST_WAIT, K_SAMPLE = range(9)
KERNEL_CLASSES = {K_DP: "hafnian_dp", K_WILLIAMSON: "williamson", K_THERMAL: "thermal_topk", K_SIGMA: "site_sigma",
                  K_PREP: "prep", K_CONTRACT: "contract", K_SAMPLE: "sample"}
HOST_CLASSES = {K_HOST_PLAN: "host_plan", K_HOST_WAIT: "host_wait"}
OUT_C64, OUT_C128 = 0, 1
(TUNE_DP_BLOCKS_PER_SM, TUNE_DP_L1_CARVEOUT, TUNE_DP_SMALL_ENTRIES, TUNE_DP_SMALL_BLOCKS, TUNE_DP_SCRATCH_MIB,
 TUNE_DP_FP64_BLOCKS, TUNE_FACTOR_THREADS, TUNE_GEMM_KERNEL, TUNE_DP_QUANTUM, TUNE_DP_HOLD, TUNE_RIGHT_PCT,
 TUNE_LEFT_PCT, TUNE_FACTOR_DUAL, TUNE_DP_ORDER) = range(14)

ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "input not positive definite",
          -4: "no convergence", -5: "size limit exceeded", -6: "allocation failed"}

# (name, restype, argtypes)
_P = C.c_void_p
_I = C.c_int
_L = C.c_int64
_D = C.c_double
SIGNATURES = {
    "bsg_create": (_I, [_I, C.POINTER(_P)]),
    "bsg_destroy": (_I, [_P]),
    "bsg_last_error": (C.c_char_p, []),
    "bsg_version": (_I, []),
    "bsg_hafnian_batched": (_I, [_P, _P, _I, _P, _I, _L, _P, _I, _P, _P]),
    "bsg_hafnian_matrices": (_I, [_P, _P, _I, _L, _I, _P, _P]),
    "bsg_site_sigma": (_I, [_P, _P, _I, _P, _I, _P, _P, _P]),
    "bsg_site_sigma_noalloc": (_I, [_P, _I, _P, _I, _P, _P, _P]),
    "bsg_first_sigma": (_I, [_P, _P, _I, _P, _P, _P, _P]),
    "bsg_build_site": (_I, [_P, _I, _P, _I, _P, _I, _I, _P, _P, _I, _I, _P, _I, _I, _I, _I, _P, _P]),
    "bsg_cut_spectra": (_I, [_P, _P, _I, _I, _I, _I, _I, _D, _P, _P, _P, _P, _P]),
    "bsg_pattern_amplitudes": (_I, [_P, _P, _P, _I, _I, _I, _P, _L, _I, _P, _P]),
    "bsg_contract_patterns": (_I, [_P, _P, _P, _I, _I, _I, _P, _L, _I, _P, _P]),
    "bsg_cut_spectrum": (_I, [_P, _P, _I, _I, _I, _I, _D, _L, _P, _P, _P, _P, _P]),
    "bsg_build_mps": (_I, [_P, _P, _I, _I, _I, _D, _D, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
    "bsg_build_mps_to_host": (_I, [_P, _P, _I, _I, _I, _D, _D, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "bsg_build_mps_batch": (_I, [_P, _I, _P, _P, _P, _P, _D, _D, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
    "bsg_build_sites": (_I, [_P, _P, _I, _I, _I, _D, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
    "bsg_profile_enable": (_I, [_P, _I]),
    "bsg_profile_read": (_I, [_P, _I, C.POINTER(_D), C.POINTER(_L), C.POINTER(_D)]),
    "bsg_profile_reset": (_I, [_P]),
    "bsg_fma_peak": (_I, [_P, _I, C.POINTER(_D), _P]),
    "bsg_gemm_tf32x3": (_I, [_P, _P, _P, _P, _I, _I, _I, _P]),
    "bsg_gemm_sliced": (_I, [_P, _P, _P, _P, _I, _I, _I, _P]),
    "bsg_tune_set": (_I, [_P, _I, _I]),
    "bsg_tune_get": (_I, [_P, _I, C.POINTER(_I)]),
    "bsg_sample": (_I, [_P, _P, _P, _I, _I, _I, _I, _P, _P, _P, _L, _I, _P, _P]),
    "bsg_profile_cut_phases": (_I, [_P, C.POINTER(_I), C.POINTER(_I), _P]),
    "bsg_profile_build_timeline": (_I, [_P, _P, _I]),
    "bsg_profile_dp_buckets": (_I, [_P, _P, _I, C.POINTER(_I), _P, _I]),
    "bsg_displacements": (_I, [_P, _P, _L, _I, _P, _P]),
    "bsg_cov_decomposition": (_I, [_P, _P, _I, _P, _D, _I, _P, _P]),
    "bsg_potrf_f64": (_I, [_P, _P, _I, _P, _P]),
    "bsg_profile_plan_phases": (_I, [_P, _P, _I]),
}


class BSGError(RuntimeError):
    pass


_lock = threading.Lock()
_lib = None


def load() -> C.CDLL:
    """Load libbsg.so (raises BSGError if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise BSGError(f"{LIB_PATH} is missing: run `python -m bosonsupremacy_gb300.build` (no CPU fallback)")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status: int, what: str) -> None:
    if status != 0:
        msg = load().bsg_last_error().decode(errors="replace")
        raise BSGError(f"{what}: {ERRORS.get(status, status)}: {msg}")


def ptr(t) -> int:
    """Device pointer of a torch tensor (None -> NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise BSGError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise BSGError("expected a contiguous tensor")
    return t.data_ptr()


def stream_ptr(stream=None) -> int:
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


class Handle:
    """Owns one bsg handle (plans, programs and scratch) for one device."""

    _per_device = {}

    def __init__(self, device: int = 0):
        lib = load()
        h = C.c_void_p()
        check(lib.bsg_create(int(device), C.byref(h)), "bsg_create")
        self._h = h
        self.device = device

    @classmethod
    def get(cls, device: int = 0) -> "Handle":
        if device not in cls._per_device:
            cls._per_device[device] = Handle(device)
        return cls._per_device[device]

    @property
    def h(self):
        return self._h

    def close(self):
        if self._h:
            load().bsg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
