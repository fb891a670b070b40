"""ctypes loader of the CPU restatement (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg use it as the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"


class EncodeParams(C.Structure):
    _fields_ = [("global_scale", C.c_uint32), ("quant_lf", C.c_uint32),
                ("x_qm_scale", C.c_uint32), ("b_qm_scale", C.c_uint32),
                ("gaborish", C.c_uint32), ("cfl", C.c_uint32)]


class LfCfl(C.Structure):
    _fields_ = [("x_factor_lf", C.c_int32), ("b_factor_lf", C.c_int32)]


class RenderParams(C.Structure):
    _fields_ = [("global_scale", C.c_uint32), ("quant_lf", C.c_uint32),
                ("x_qm_scale", C.c_uint32), ("b_qm_scale", C.c_uint32),
                ("gaborish", C.c_uint32), ("epf_iters", C.c_uint32),
                ("x_factor_lf", C.c_int32), ("b_factor_lf", C.c_int32)]


def build() -> Path:
    """Builds liboracle.so with the committed Makefile (gcc, no GPU)."""
    res = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    return LIB


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        lib = C.CDLL(str(LIB))
        f, i, p = C.c_float, C.c_int, C.c_void_p
        for name in ("orc_cbrt_core", "orc_cbrt_perceptual", "orc_srgb_to_linear",
                     "orc_linear_to_srgb"):
            getattr(lib, name).restype = f
            getattr(lib, name).argtypes = [f]
        lib.orc_hf_multiplier.restype = f
        lib.orc_hf_multiplier.argtypes = [C.c_uint32, C.c_uint32]
        lib.orc_bias_adjust.restype = f
        lib.orc_bias_adjust.argtypes = [C.c_int32, f, f]
        lib.orc_scale_f.restype = f
        lib.orc_scale_f.argtypes = [i, i]
        lib.orc_gaborish_w.argtypes = [p, i, i, f, f, p]
        lib.orc_encode.restype = i
        lib.orc_encode.argtypes = [p, i, i, i, p, p, p, p, p, p, p, p, p, p, p]
        lib.orc_reconstruct.restype = i
        lib.orc_reconstruct.argtypes = [i, i, p, p, p, p, p, p, p, p, i, i, p]
        lib.orc_select_blocks.restype = i
        lib.orc_select_blocks.argtypes = [p, i, i, i, p, p, p]
        lib.orc_ssim2.restype = i
        lib.orc_ssim2.argtypes = [p, p, i, i, p, p, p]
        lib.orc_perceptual_add_noise.argtypes = [p, p, p, i, f, C.c_uint32]
        lib.orc_perceptual_synthetic.argtypes = [i, i, C.c_uint32, p, p, p]
        for name in ("orc_dct_2d", "orc_idct_2d"):
            getattr(lib, name).argtypes = [p, i, i]
        for name in ("orc64_dct_2d", "orc64_idct_2d"):
            getattr(lib, name).argtypes = [p, i, i, p]
        lib.orc64_encode_transform.restype = i
        lib.orc64_encode_transform.argtypes = [p, i, i, i, p, i, p, p, p]
        lib.orc64_reconstruct.restype = i
        lib.orc64_reconstruct.argtypes = [i, i, p, p, p, p, p, p, p, p, i, p]
        lib.orc64_ssim2.restype = i
        lib.orc64_ssim2.argtypes = [p, p, p, p, i, i, p, p]
        lib.orc_special_block.restype = i
        lib.orc_special_block.argtypes = [i, p, p, p]
        _lib = lib
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def select_blocks(rgb: np.ndarray, *, global_scale: int, quant_lf: int = 16,
                  x_qm_scale: int = 2, b_qm_scale: int = 2, gaborish: bool = False,
                  bits: int | None = None):
    """orc_select_blocks: returns (rc, block map uint8 [bh, bw], candidates scored)."""
    lib = load()
    h, w = rgb.shape[:2]
    if bits is None:
        bits = 8 if rgb.dtype == np.uint8 else 16
    rgb = np.ascontiguousarray(rgb)
    out = np.zeros(((h + 7) // 8, (w + 7) // 8), np.uint8)
    prm = EncodeParams(global_scale, quant_lf, x_qm_scale, b_qm_scale, int(gaborish), 1)
    scored = C.c_int64()
    rc = lib.orc_select_blocks(rgb.ctypes.data, w, h, bits, C.byref(prm), out.ctypes.data,
                               C.byref(scored))
    return rc, out, scored.value


def encode(rgb: np.ndarray, block_map: np.ndarray, hf_mul: np.ndarray, *, global_scale: int,
           quant_lf: int = 16, x_qm_scale: int = 2, b_qm_scale: int = 2, gaborish: bool = False,
           cfl: bool = True, bits: int | None = None, stages: bool = False):
    """orc_encode: returns (rc, dict of outputs)."""
    lib = load()
    h, w = rgb.shape[:2]
    bw, bh = (w + 7) // 8, (h + 7) // 8
    tw, th = (bw + 7) // 8, (bh + 7) // 8
    if bits is None:
        bits = 8 if rgb.dtype == np.uint8 else 16
    rgb = np.ascontiguousarray(rgb)
    out = {
        "qcoeff": np.zeros((3, bh * 8, bw * 8), np.int32),
        "lf": np.zeros((3, bh, bw), np.int32),
        "cfl_x": np.zeros((th, tw), np.int8),
        "cfl_b": np.zeros((th, tw), np.int8),
    }
    if stages:
        out["xyb"] = np.zeros((3, h, w), np.float32)
        out["pre"] = np.zeros((3, h, w), np.float32)
        out["coeff"] = np.zeros((3, bh * 8, bw * 8), np.float32)
    lfc = LfCfl()
    p = EncodeParams(global_scale, quant_lf, x_qm_scale, b_qm_scale, int(gaborish), int(cfl))
    bm = np.ascontiguousarray(block_map, np.uint8)
    hm = np.ascontiguousarray(hf_mul, np.uint32)
    rc = lib.orc_encode(rgb.ctypes.data, w, h, bits, bm.ctypes.data, hm.ctypes.data, C.byref(p),
                        _ptr(out.get("xyb")), _ptr(out.get("pre")), _ptr(out.get("coeff")),
                        out["qcoeff"].ctypes.data, out["lf"].ctypes.data,
                        out["cfl_x"].ctypes.data, out["cfl_b"].ctypes.data, C.byref(lfc))
    out["lf_factors"] = (lfc.x_factor_lf, lfc.b_factor_lf)
    return rc, out


def reconstruct(w: int, h: int, block_map, hf_mul, sharpness, plan: dict, *, global_scale: int,
                quant_lf: int = 16, x_qm_scale: int = 2, b_qm_scale: int = 2,
                gaborish: bool = False, epf_iters: int = 0, out_kind: int = 2, bits: int = 8):
    lib = load()
    p = RenderParams(global_scale, quant_lf, x_qm_scale, b_qm_scale, int(gaborish), epf_iters,
                     int(plan["lf_factors"][0]), int(plan["lf_factors"][1]))
    out = (np.zeros((h, w, 3), np.uint8) if out_kind == 2 else np.zeros((3, h, w), np.float32))
    arrs = [np.ascontiguousarray(block_map, np.uint8), np.ascontiguousarray(hf_mul, np.uint32),
            np.ascontiguousarray(sharpness, np.uint8),
            np.ascontiguousarray(plan["qcoeff"], np.int32),
            np.ascontiguousarray(plan["lf"], np.int32),
            np.ascontiguousarray(plan["cfl_x"], np.int8),
            np.ascontiguousarray(plan["cfl_b"], np.int8)]
    rc = lib.orc_reconstruct(w, h, *[a.ctypes.data for a in arrs], C.byref(p), out_kind, bits,
                             out.ctypes.data)
    return rc, out


def ssim2(ref: np.ndarray, cand: np.ndarray):
    """orc_ssim2 on linear float32 [3, H, W] planes: (score, raw_error, terms)."""
    lib = load()
    ref = np.ascontiguousarray(ref, np.float32)
    cand = np.ascontiguousarray(cand, np.float32)
    _, h, w = ref.shape
    ra = (C.c_void_p * 3)(*[ref[c].ctypes.data for c in range(3)])
    ca = (C.c_void_p * 3)(*[cand[c].ctypes.data for c in range(3)])
    sc, raw = C.c_double(), C.c_double()
    terms = np.zeros(6 * 18, np.float64)
    n = lib.orc_ssim2(ra, ca, w, h, C.byref(sc), C.byref(raw), terms.ctypes.data)
    return sc.value, raw.value, terms[: max(n, 0) * 18]


def perceptual_pair(w: int, h: int, seed: int, amp: float, noise_seed: int):
    """The reference's perceptual test fixtures (synthetic + add_noise)."""
    lib = load()
    a = np.zeros((3, h, w), np.float32)
    lib.orc_perceptual_synthetic(w, h, seed, a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data)
    b = a.copy()
    lib.orc_perceptual_add_noise(b[0].ctypes.data, b[1].ctypes.data, b[2].ctypes.data, w * h,
                                 C.c_float(amp), noise_seed)
    return a, b


# ---- FP64 truth (oracle_fp64.cpp): the same algorithm in f64 throughout ----

def dct_2d(block: np.ndarray, f64: bool = False) -> np.ndarray:
    """DCT_2D of a rows x cols block into the landscape layout (f32 butterflies
    of the restatement, or the f64 truth with `f64`)."""
    lib = load()
    rows, cols = block.shape
    shape = (rows, cols) if cols > rows else (cols, rows)
    if f64:
        src = np.ascontiguousarray(block, np.float64)
        out = np.zeros(shape, np.float64)
        lib.orc64_dct_2d(src.ctypes.data, rows, cols, out.ctypes.data)
        return out
    work = np.ascontiguousarray(block, np.float32).copy()
    lib.orc_dct_2d(work.ctypes.data, rows, cols)
    return work.reshape(shape)


def idct_2d(coef: np.ndarray, rows: int, cols: int, f64: bool = False) -> np.ndarray:
    """IDCT_2D of landscape coefficients into rows x cols samples."""
    lib = load()
    if f64:
        src = np.ascontiguousarray(coef, np.float64)
        out = np.zeros((rows, cols), np.float64)
        lib.orc64_idct_2d(src.ctypes.data, rows, cols, out.ctypes.data)
        return out
    work = np.ascontiguousarray(coef, np.float32).copy()
    lib.orc_idct_2d(work.ctypes.data, rows, cols)
    return work.reshape(rows, cols)


def fp64_encode_transform(rgb: np.ndarray, block_map: np.ndarray, *, gaborish: bool,
                          bits: int | None = None):
    """orc64_encode_transform: (rc, xyb, preconditioned planes, coefficient image), f64."""
    lib = load()
    h, w = rgb.shape[:2]
    bw, bh = (w + 7) // 8, (h + 7) // 8
    if bits is None:
        bits = 8 if rgb.dtype == np.uint8 else 16
    rgb = np.ascontiguousarray(rgb)
    xyb = np.zeros((3, h, w), np.float64)
    pre = np.zeros((3, h, w), np.float64)
    coeff = np.zeros((3, bh * 8, bw * 8), np.float64)
    bm = np.ascontiguousarray(block_map, np.uint8)
    rc = lib.orc64_encode_transform(rgb.ctypes.data, w, h, bits, bm.ctypes.data, int(gaborish),
                                    xyb.ctypes.data, pre.ctypes.data, coeff.ctypes.data)
    return rc, xyb, pre, coeff


def fp64_reconstruct(w: int, h: int, block_map, hf_mul, sharpness, plan: dict, *,
                     global_scale: int, quant_lf: int = 16, x_qm_scale: int = 2,
                     b_qm_scale: int = 2, gaborish: bool = False, epf_iters: int = 0,
                     out_kind: int = 1):
    """orc64_reconstruct: (rc, [3, h, w] f64): out_kind 1 linear sRGB, 0 XYB
    after restoration, 4 XYB before restoration."""
    lib = load()
    p = RenderParams(global_scale, quant_lf, x_qm_scale, b_qm_scale, int(gaborish), epf_iters,
                     int(plan["lf_factors"][0]), int(plan["lf_factors"][1]))
    out = np.zeros((3, h, w), np.float64)
    arrs = [np.ascontiguousarray(block_map, np.uint8), np.ascontiguousarray(hf_mul, np.uint32),
            np.ascontiguousarray(sharpness, np.uint8),
            np.ascontiguousarray(plan["qcoeff"], np.int32),
            np.ascontiguousarray(plan["lf"], np.int32),
            np.ascontiguousarray(plan["cfl_x"], np.int8),
            np.ascontiguousarray(plan["cfl_b"], np.int8)]
    rc = lib.orc64_reconstruct(w, h, *[a.ctypes.data for a in arrs], C.byref(p), out_kind,
                               out.ctypes.data)
    return rc, out


def fp64_ssim2(ref: np.ndarray, cand: np.ndarray):
    """orc64_ssim2 on linear [3, H, W] planes (f32 or f64): (score, terms)."""
    lib = load()
    _, h, w = ref.shape

    def planes(a):
        if a.dtype == np.float64:
            a = np.ascontiguousarray(a)
            return None, (C.c_void_p * 3)(*[a[c].ctypes.data for c in range(3)]), a
        a = np.ascontiguousarray(a, np.float32)
        return (C.c_void_p * 3)(*[a[c].ctypes.data for c in range(3)]), None, a

    r32, r64, _ra = planes(ref)
    c32, c64, _ca = planes(cand)
    sc = C.c_double()
    terms = np.zeros(6 * 18, np.float64)
    n = lib.orc64_ssim2(r32, c32, r64, c64, w, h, C.byref(sc), terms.ctypes.data)
    return sc.value, terms[: max(n, 0) * 18]


SPECIAL_KINDS = {"dct2x2": 1, "hornuss": 2, "dct4x4": 3, "dct8x4": 4, "dct4x8": 5,
                 "afv0": 6, "afv1": 7, "afv2": 8, "afv3": 9}


def special_block(kind: int, coef: np.ndarray, afv_basis=None) -> np.ndarray:
    """orc_special_block: a dequantized 8x8 coefficient block (float32 [8, 8],
    row-major, LLF at [0, 0]) to its 8x8 samples; afv_basis is Table I.11
    ([16, 16] f64), needed for the AFV kinds 6..9."""
    lib = load()
    c = np.ascontiguousarray(coef, np.float32).reshape(8, 8)
    out = np.zeros((8, 8), np.float32)
    basis = None if afv_basis is None else np.ascontiguousarray(afv_basis, np.float64)
    rc = lib.orc_special_block(kind, c.ctypes.data, _ptr(basis), out.ctypes.data)
    if rc:
        raise ValueError(f"orc_special_block kind {kind}: {rc}")
    return out
