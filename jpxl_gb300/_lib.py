"""ctypes binding of ``libjpxlg.so`` (the C ABI declared in include/jpxlg.h).

The library is the product: there is no CPU fallback.  ``load()`` raises if
the shared object is missing or fails to load, so a caller on a machine with a
GPU that has not built the library (``__graft_entry__.build()``) fails loudly
instead of silently running something else.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libjpxlg.so"

# Every symbol include/jpxlg.h declares, with its ctypes signature.
_P = C.c_void_p
_I = C.c_int
_U32 = C.c_uint32
SIGNATURES: dict[str, tuple] = {
    "jpxlg_ctx_create": (_I, [_I, _U32, C.POINTER(_P)]),
    "jpxlg_ctx_destroy": (_I, [_P]),
    "jpxlg_ctx_set_stream": (_I, [_P, _P]),
    "jpxlg_ctx_stream": (_P, [_P]),
    "jpxlg_ctx_synchronize": (_I, [_P]),
    "jpxlg_last_error": (C.c_char_p, [_P]),
    "jpxlg_ctx_launches": (C.c_uint64, [_P]),
    "jpxlg_ctx_cfl_fallbacks": (_U32, [_P]),
    "jpxlg_stage_timing": (_I, [_P, _I]),
    "jpxlg_stage_times": (_I, [_P, _P, _P, _I]),
    "jpxlg_layout_create": (_I, [_P, _I, _I, _P, _P, _P, C.POINTER(_P)]),
    "jpxlg_layout_destroy": (_I, [_P]),
    "jpxlg_layout_dims": (_I, [_P, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)]),
    "jpxlg_encode_transform": (_I, [_P, _P, _P, _I, _P, _P, _U32]),
    "jpxlg_encode_stages": (_I, [_P, _P, _P, _I, _P, _P, _P, _P]),
    "jpxlg_diag_special_blocks": (_I, [_P, _I, _P, _I, _P, _U32]),
    "jpxlg_tune_set": (_I, [_I, _I]),
    "jpxlg_tune_get": (_I, [_I]),
    "jpxlg_reconstruct": (_I, [_P, _P, _P, _P, _I, _I, _P, _U32]),
    "jpxlg_ssim2_ref_create": (_I, [_P, _P, _I, _I, _U32, C.POINTER(_P)]),
    "jpxlg_ssim2_ref_destroy": (_I, [_P]),
    "jpxlg_ssim2_score": (_I, [_P, _P, _P, _U32, _P, _P, _P]),
    "jpxlg_score_pair": (_I, [_P, _P, _P, _I, _I, _U32, _P]),
    "jpxlg_probe": (_I, [_P, _P, _P, _P, _I, _P, _U32, _P]),
    "jpxlg_ssim2_score_static": (_I, [_P, _P, _P, _P]),
    "jpxlg_select_blocks": (_I, [_P, _I, _I, _P, _I, _P, _P, _U32]),
    "jpxlg_ctx_cover_fallbacks": (_U32, [_P]),
    "jpxlg_batch_create": (_I, [_P, _I, _P, _I, C.POINTER(_P)]),
    "jpxlg_batch_run": (_I, [_P, _P, _P, _U32]),
    "jpxlg_batch_destroy": (_I, [_P]),
    "jpxlg_batch_probe": (_I, [_P, _I, _P, _P]),
    "jpxlg_symbols_open": (_I, [_P, C.c_size_t, C.c_size_t, _U32, C.POINTER(_P)]),
    "jpxlg_symbols_read": (_I, [_P, _U32, C.POINTER(_U32)]),
    "jpxlg_symbols_read_many": (_I, [_P, _P, C.c_size_t, _P]),
    "jpxlg_symbols_set_dist_multiplier": (_I, [_P, _U32]),
    "jpxlg_symbols_finish": (_I, [_P]),
    "jpxlg_symbols_bits_read": (C.c_size_t, [_P]),
    "jpxlg_symbols_destroy": (_I, [_P]),
    "jpxlg_codestream_open": (_I, [_P, C.c_size_t, C.POINTER(_P)]),
    "jpxlg_codestream_open_limits": (_I, [_P, C.c_size_t, _P, C.POINTER(_P)]),
    "jpxlg_codestream_last_error": (C.c_char_p, []),
    "jpxlg_codestream_info": (_I, [_P, _P]),
    "jpxlg_codestream_blocks": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "jpxlg_codestream_coefficients": (_I, [_P, _P]),
    "jpxlg_codestream_channel": (_I, [_P, _U32, _P]),
    "jpxlg_codestream_extra": (_I, [_P, _U32, _P]),
    "jpxlg_codestream_destroy": (_I, [_P]),
    "jpxlg_codestream_render": (_I, [_P, _P, _I, _P, _U32]),
    "jpxlg_decode_batch_create": (_I, [_P, _I, _P, _I, _U32, _I, C.POINTER(_P)]),
    "jpxlg_decode_batch_run": (_I, [_P, _P, _P, _U32]),
    "jpxlg_decode_batch_destroy": (_I, [_P]),
}


class Params(C.Structure):
    """jpxlg_params (include/jpxlg.h)."""

    _fields_ = [
        ("global_scale", C.c_uint32),
        ("quant_lf", C.c_uint32),
        ("x_qm_scale", C.c_uint32),
        ("b_qm_scale", C.c_uint32),
        ("gaborish", C.c_uint32),
        ("epf_iters", C.c_uint32),
        ("cfl", C.c_uint32),
        ("precision", C.c_uint32),
    ]


class BatchItemStruct(C.Structure):
    """jpxlg_batch_item (include/jpxlg.h)."""

    _fields_ = [
        ("layout", C.c_void_p),
        ("ref", C.c_void_p),
        ("rgb", C.c_void_p),
        ("bits", C.c_int),
        ("params", Params),
    ]


class PlanStruct(C.Structure):
    """jpxlg_plan (include/jpxlg.h)."""

    _fields_ = [
        ("qcoeff", C.c_void_p),
        ("lf", C.c_void_p),
        ("cfl_x", C.c_void_p),
        ("cfl_b", C.c_void_p),
        ("lf_factors", C.c_int32 * 2),
    ]


_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Loads libjpxlg.so once and binds every declared symbol."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build the CUDA library first (python -c "
            "'import __graft_entry__ as g; g.build()'); there is no CPU fallback"
        )
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
