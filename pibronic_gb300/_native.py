"""ctypes binding of ``libpibronic_gb300.so`` (the C ABI declared in ``include/pibronic_gb300.h``).

The library is loaded lazily on first use.  There is no CPU fallback: if the library is missing,
cannot be loaded, or no CUDA device is present, every compute call raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_LOCK = threading.Lock()
_LIB = None

PBR_OK, PBR_ERR_ARG, PBR_ERR_CUDA, PBR_ERR_UNSUPPORTED, PBR_ERR_NONFINITE = 0, 1, 2, 3, 4
PBR_ERR_CAPACITY = 5
_STATUS_TEXT = {
    PBR_ERR_ARG: "invalid argument",
    PBR_ERR_CUDA: "CUDA error",
    PBR_ERR_UNSUPPORTED: "unsupported sizes for the compiled kernels",
    PBR_ERR_NONFINITE: "non-finite result",
    PBR_ERR_CAPACITY: "request exceeds a fixed capacity of the library",
}

#: every symbol declared in include/pibronic_gb300.h
EXPORTED = (
    "pbr_sample_eval", "pbr_sample_q", "pbr_eval_q", "pbr_eval_q_f32",
    "pbr_o_matrix", "pbr_scale_o_matrices", "pbr_scaling_factors", "pbr_divide_o_matrix", "pbr_denominator",
    "pbr_coupling_eigh", "pbr_numerator",
    "pbr_reduce_terms", "pbr_reduce_jackknife", "pbr_reduce_blocks", "pbr_fma_probe",
    "pbr_reduce_terms_static", "pbr_reduce_terms_static_max_samples",
    "pbr_flow_prepare", "pbr_flow_apply", "pbr_flow_layer_forward", "pbr_flow_layer_backward",
    "pbr_flow_tc_packed_bytes", "pbr_flow_tc_pack", "pbr_flow_tc_forward",
    "pbr_gemm_tn_acc", "pbr_gemm_tn_scratch", "pbr_colsum", "pbr_flow_base", "pbr_flow_weights",
    "pbr_adam", "pbr_batch_blob_bytes", "pbr_batch_pack", "pbr_sample_eval_batch", "pbr_batch_groups",
    "pbr_reduce_terms_segments", "pbr_reduce_jackknife_segments", "pbr_reduce_segments_scratch",
    "pbr_tc_gemm", "pbr_tc_mma_rate", "pbr_tc_potential_dims", "pbr_tc_potential_packed_floats", "pbr_tc_pack_potential",
    "pbr_tc_potential",
    "pbr_sample_eval_tc_scratch", "pbr_sample_eval_tc", "pbr_eval_q_tc", "pbr_version",
)


class PbrModel(C.Structure):
    """Mirror of ``pbr_model``."""
    _fields_ = [
        ("A", C.c_int32), ("A_rho", C.c_int32), ("n_fill_rho", C.c_int32), ("N", C.c_int32),
        ("P", C.c_int32), ("K", C.c_int32), ("precision", C.c_int32), ("variant", C.c_int32),
        ("tau", C.c_double), ("delta_beta", C.c_double), ("log_c0", C.c_double),
        ("vib_cs", C.c_void_p), ("vib_th", C.c_void_p), ("vib_c", C.c_void_p),
        ("vib_d", C.c_void_p), ("vib_e", C.c_void_p), ("vib_l", C.c_void_p),
        ("vib_qq", C.c_void_p), ("rho_cs", C.c_void_p), ("rho_th", C.c_void_p),
        ("rho_c", C.c_void_p), ("rho_d", C.c_void_p), ("ring_chol", C.c_void_p),
        ("src_cdf", C.c_void_p),
    ]


class PbrFlowLayer(C.Structure):
    """Mirror of ``pbr_flow_layer``."""
    _fields_ = [("D", C.c_int32), ("I", C.c_int32), ("J", C.c_int32), ("H", C.c_int32),
                ("idx_a", C.c_void_p), ("idx_b", C.c_void_p), ("W1", C.c_void_p), ("b1", C.c_void_p),
                ("W2", C.c_void_p), ("b2", C.c_void_p), ("W3", C.c_void_p), ("b3", C.c_void_p)]


class PbrFlowSave(C.Structure):
    """Mirror of ``pbr_flow_save``."""
    _fields_ = [("ya", C.c_void_p), ("h1", C.c_void_p), ("h2", C.c_void_p), ("s", C.c_void_p),
                ("yb", C.c_void_p)]


class PbrOutputs(C.Structure):
    """Mirror of ``pbr_outputs``."""
    _fields_ = [
        ("s_rho", C.c_void_p), ("s_g", C.c_void_p), ("s_gp", C.c_void_p), ("s_gm", C.c_void_p),
        ("g_coef", C.c_void_p), ("log_scale", C.c_void_p), ("q_out", C.c_void_p),
        ("src_out", C.c_void_p), ("status", C.c_void_p),
    ]


def lib_path():
    here = os.path.dirname(os.path.abspath(__file__))
    return os.path.join(here, "_lib", "libpibronic_gb300.so")


def _declare(lib):
    vp, i32, i64, u64, f64 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_double
    sig = {
        "pbr_sample_eval": (C.c_int, [C.POINTER(PbrModel), u64, u64, i64, C.POINTER(PbrOutputs), vp]),
        "pbr_sample_q": (C.c_int, [C.POINTER(PbrModel), u64, u64, i64, vp, vp, vp]),
        "pbr_eval_q": (C.c_int, [C.POINTER(PbrModel), vp, i64, C.POINTER(PbrOutputs), vp]),
        "pbr_eval_q_f32": (C.c_int, [C.POINTER(PbrModel), vp, i64, C.POINTER(PbrOutputs), vp]),
        "pbr_o_matrix": (C.c_int, [vp, i64, i32, i32, i32, vp, vp, vp, vp, i32, vp, vp]),
        "pbr_scale_o_matrices": (C.c_int, [vp, i32, vp, i32, i64, i32, vp, vp]),
        "pbr_scaling_factors": (C.c_int, [vp, i32, vp, i32, i64, i32, vp, vp, vp, vp]),
        "pbr_divide_o_matrix": (C.c_int, [vp, i32, i64, i32, vp, vp]),
        "pbr_denominator": (C.c_int, [vp, i64, i32, i32, vp, vp]),
        "pbr_coupling_eigh": (C.c_int, [vp, i64, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp]),
        "pbr_numerator": (C.c_int, [vp, vp, vp, i64, i32, i32, f64, vp, vp, vp]),
        "pbr_reduce_terms": (C.c_int, [vp, vp, vp, vp, i64, f64, vp, vp, vp]),
        "pbr_reduce_jackknife": (C.c_int, [vp, vp, vp, vp, i64, f64, f64, vp, vp, vp, vp]),
        "pbr_reduce_blocks": (i64, [i64]),
        "pbr_fma_probe": (C.c_int, [vp, i32, i32, C.POINTER(f64), vp]),
        "pbr_reduce_terms_static": (C.c_int, [vp, vp, vp, vp, i64, f64, vp, vp]),
        "pbr_reduce_terms_static_max_samples": (i64, []),
        "pbr_flow_prepare": (C.c_int, [vp, i64, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp]),
        "pbr_flow_apply": (C.c_int, [vp, vp, vp, i64, i32, i32, i32, vp, vp, vp]),
        "pbr_flow_layer_forward": (C.c_int, [C.POINTER(PbrFlowLayer), i32, i64, vp, vp,
                                             C.POINTER(PbrFlowSave), vp]),
        "pbr_flow_layer_backward": (C.c_int, [C.POINTER(PbrFlowLayer), i64, vp, vp,
                                              C.POINTER(PbrFlowSave), vp, vp, vp, vp]),
        "pbr_flow_tc_packed_bytes": (i64, [i32, i32, i32, i32]),
        "pbr_flow_tc_pack": (C.c_int, [C.POINTER(PbrFlowLayer), vp, vp]),
        "pbr_flow_tc_forward": (C.c_int, [C.POINTER(PbrFlowLayer), vp, i64, vp, vp, vp, vp]),
        "pbr_gemm_tn_acc": (C.c_int, [vp, vp, i64, i32, i32, C.c_float, vp, vp, vp, vp]),
        "pbr_gemm_tn_scratch": (i64, [i64, i32, i32]),
        "pbr_colsum": (C.c_int, [vp, i64, i32, vp, vp]),
        "pbr_flow_base": (C.c_int, [vp, vp, i64, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp]),
        "pbr_flow_weights": (C.c_int, [vp, vp, vp, vp, i64, vp, vp]),
        "pbr_adam": (C.c_int, [vp, vp, vp, vp, i64, C.c_float, C.c_float, C.c_float, C.c_float, vp, vp]),
        "pbr_batch_blob_bytes": (i64, [i32]),
        "pbr_batch_pack": (C.c_int, [vp, vp, vp, vp, vp, i32, vp, i32, vp]),
        "pbr_sample_eval_batch": (C.c_int, [vp, vp, vp]),
        "pbr_batch_groups": (i32, [vp]),
        "pbr_reduce_terms_segments": (C.c_int, [vp, vp, vp, vp, vp, i32, vp, vp, vp, vp]),
        "pbr_reduce_jackknife_segments": (C.c_int, [vp, vp, vp, vp, vp, i32, vp, vp, vp, vp, vp, vp]),
        "pbr_reduce_segments_scratch": (i64, [i32]),
        "pbr_tc_gemm": (C.c_int, [i32, vp, vp, vp, i32, i32, i32, vp, vp]),
        "pbr_tc_potential_dims": (C.c_int, [i32, i32, C.POINTER(i32), C.POINTER(i32)]),
        "pbr_tc_potential_packed_floats": (i64, [i32, i32]),
        "pbr_tc_mma_rate": (C.c_int, [i32, i32, i32, i32, i32, i32, vp, C.POINTER(f64), C.POINTER(f64), vp]),
        "pbr_tc_pack_potential": (C.c_int, [vp, vp, vp, i32, i32, i32, vp, vp]),
        "pbr_tc_potential": (C.c_int, [vp, i64, i32, i32, i32, vp, vp, vp, vp]),
        "pbr_sample_eval_tc_scratch": (i64, [C.POINTER(PbrModel), i64]),
        "pbr_sample_eval_tc": (C.c_int, [C.POINTER(PbrModel), u64, u64, i64, C.POINTER(PbrOutputs), vp, i64, vp]),
        "pbr_eval_q_tc": (C.c_int, [C.POINTER(PbrModel), vp, i64, C.POINTER(PbrOutputs), vp, i64, vp]),
        "pbr_version": (C.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


class _StrictLibrary:
    """The ctypes library with every declared entry point checked for its argument count: ctypes
    itself passes surplus arguments on silently, which would turn a stale call into a wrong
    pointer (a stream handle, say) inside the library."""

    def __init__(self, lib):
        self._lib = lib
        self._cache = {}

    def __getattr__(self, name):
        fn = self._cache.get(name)
        if fn is None:
            raw = getattr(self._lib, name)
            nargs = len(raw.argtypes) if raw.argtypes is not None else None

            def fn(*args, _raw=raw, _n=nargs, _name=name):
                if _n is not None and len(args) != _n:
                    raise TypeError(f"{_name} takes {_n} arguments ({len(args)} given)")
                return _raw(*args)

            fn.raw = raw
            self._cache[name] = fn
        return fn


def load(path=None):
    """Load (once) and return the ctypes library handle; raises RuntimeError when unavailable."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = path or lib_path()
        if not os.path.exists(path):
            raise RuntimeError(
                f"pibronic_gb300 CUDA library not built ({path}); run pibronic_gb300.build.build()")
        lib = C.CDLL(path)
        missing = [s for s in EXPORTED if not hasattr(lib, s)]
        if missing:
            raise RuntimeError(f"{path} lacks symbols {missing}")
        _declare(lib)
        _LIB = _StrictLibrary(lib)
        return _LIB


def check(status, what):
    """Map a non-zero status to the reference's exception types (AssertionError for argument
    and shape problems, RuntimeError for device failures)."""
    if status == PBR_OK:
        return
    text = _STATUS_TEXT.get(status, f"status {status}")
    if status in (PBR_ERR_ARG, PBR_ERR_UNSUPPORTED):
        raise AssertionError(f"{what}: {text}")
    raise RuntimeError(f"{what}: {text}")


def require_cuda():
    """The product path runs on the GPU only; fail loudly otherwise."""
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("pibronic_gb300 needs a CUDA device: there is no CPU fallback")
    return torch


def ptr(t):
    """Device (or host) address of a torch tensor, or None."""
    return None if t is None else C.c_void_p(t.data_ptr())


def stream_handle(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)
