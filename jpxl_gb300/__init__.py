"""jpxl_gb300 — the lossy VarDCT pixel path and SSIMULACRA2 of JPXL on GB300.

Host-side mirror of the reference's entry points for this path, over the C
ABI of ``libjpxlg.so`` (include/jpxlg.h):

=============================  ==================================================
this package                   reference (JPXL, crates/...)
=============================  ==================================================
``EncodeRequest``              jpxl-encode-policy request.rs:855 EncodeRequest
``Layout``                     a validated cover: plan.rs:239 varblocks + hf_mul,
                               :318 SharpnessGrid
``encode_transform``           policy lib.rs:555 build_pixel_plan's transform and
                               quantization (source.rs:226/:355, gaborish.rs:218,
                               lib.rs:3437 estimate_cfl, :3237 quantize)
``select_blocks``              jpxl-encode-policy lib.rs:5260 select_blocks (the
                               hierarchical cover, fixed quantizer, AQ off)
``PlanRenderer.render``        jpxl-plan-render lib.rs:680 render /
                               render_linear_at_depth_with
``PrecomputedReference``       jpxl-perceptual reference.rs:90
``Ssimulacra2.score``          jpxl-perceptual ssimulacra2.rs:79
``score_pair``                 jpxl-perceptual lib.rs:195
``Context.probe``              jpxl-perceptual evaluator.rs:243 evaluate_with
``BatchProbe``                 the candidate sweep of search_frame_perceptual
                               (quality.rs:2405) over evaluate (evaluator.rs:295),
                               as one CUDA graph
``quality.search``             search_frame_perceptual's baseline solve
                               (quality.rs:1775) over BatchProbe rounds
``Codestream``                 jpxl-decode decode.rs:400 up to the frame content
``open_codestreams``           many Codestreams parsed on host threads at once
``DecodeBatch``                a loop of decode.rs:400 decode calls as one graph
=============================  ==================================================

Arrays are numpy (host memory) unless stated; the ``*_device`` variants take
integer device pointers (e.g. ``torch.Tensor.data_ptr()``) and queue work on
the context's stream without synchronizing.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import BatchItemStruct, Params, PlanStruct

MEM_HOST = 0
MEM_DEVICE = 1
OUT_XYB = 0
OUT_LINEAR = 1
OUT_SRGB8 = 2
OUT_LINEAR_DEPTH = 3

# Table I.1 DctSelect values of the plain DCT shapes this path carries.
DCT8, DCT16, DCT32 = 0, 4, 5
DCT16X8, DCT8X16, DCT32X8, DCT8X32, DCT32X16, DCT16X32 = 6, 7, 8, 9, 10, 11
SHAPES = {
    DCT8: (1, 1), DCT16: (2, 2), DCT32: (4, 4), DCT16X8: (2, 1), DCT8X16: (1, 2),
    DCT32X8: (4, 1), DCT8X32: (1, 4), DCT32X16: (4, 2), DCT16X32: (2, 4),
}
ORIGIN = 0x80

# JPXLG_STAGE_* order (include/jpxlg.h).
STAGES = ("xyb", "precondition", "fdct_luma", "cfl", "quant_chroma", "render_varblocks",
          "gaborish", "epf", "colour", "ssim", "ssim_rows", "ssim_col_ripple", "ssim_col_out")


# jpxlg_params.precision (include/jpxlg.h JPXLG_PRECISION_*)
PRECISIONS = {"fp32": 0, "bf16x3": 1, "bf16x6": 2}


class JpxlError(RuntimeError):
    """A non-zero jpxlg_status; ``code`` is the status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"jpxlg status {code}: {message}")
        self.code = code


@dataclass
class EncodeRequest:
    """The request fields the transform path reads (request.rs:855)."""

    global_scale: int = 32768
    quant_lf: int = 16
    x_qm_scale: int = 2
    b_qm_scale: int = 2
    gaborish: bool = False
    epf_iters: int = 0
    cfl: bool = True
    # How the DCTs run: "fp32" (the reference's arithmetic, bit-exact),
    # "bf16x3" or "bf16x6" (split-precision contractions on the tensor cores).
    precision: str = "fp32"

    @classmethod
    def with_global_scale(cls, gs: int, **kw) -> "EncodeRequest":
        """jpxl lib.rs:561 Encoder::with_global_scale (fixed quantizer)."""
        return cls(global_scale=gs, **kw)

    def _struct(self) -> Params:
        return Params(self.global_scale, self.quant_lf, self.x_qm_scale, self.b_qm_scale,
                      int(bool(self.gaborish)), self.epf_iters, int(bool(self.cfl)),
                      PRECISIONS[self.precision])


@dataclass
class Plan:
    """The quantized half of a plan (plan.rs:434/:519/:251, LF correlation)."""

    qcoeff: np.ndarray          # int32 [3, 8*bh, 8*bw] coefficient image
    lf: np.ndarray              # int32 [3, bh, bw]
    cfl_x: np.ndarray           # int8 [th, tw]
    cfl_b: np.ndarray           # int8 [th, tw]
    lf_factors: tuple = (128, 128)

    def _struct(self) -> PlanStruct:
        s = PlanStruct()
        s.qcoeff = self.qcoeff.ctypes.data
        s.lf = self.lf.ctypes.data
        s.cfl_x = self.cfl_x.ctypes.data
        s.cfl_b = self.cfl_b.ctypes.data
        s.lf_factors[0] = int(self.lf_factors[0])
        s.lf_factors[1] = int(self.lf_factors[1])
        return s


class Context:
    """A device context: tables, workspace and a CUDA stream (jpxlg_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        rc = self.lib.jpxlg_ctx_create(device, 0, C.byref(h))
        if rc:
            raise JpxlError(rc, "jpxlg_ctx_create failed (no sm_103 device?)")
        self.handle = h

    def check(self, rc: int) -> None:
        if rc:
            raise JpxlError(rc, self.lib.jpxlg_last_error(self.handle).decode())

    def close(self) -> None:
        if self.handle:
            self.lib.jpxlg_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return int(self.lib.jpxlg_ctx_stream(self.handle) or 0)

    def set_stream(self, stream: int | None) -> None:
        self.check(self.lib.jpxlg_ctx_set_stream(self.handle, C.c_void_p(stream or 0)))

    def synchronize(self) -> None:
        self.check(self.lib.jpxlg_ctx_synchronize(self.handle))

    @property
    def launches(self) -> int:
        return int(self.lib.jpxlg_ctx_launches(self.handle))

    @property
    def cfl_fallbacks(self) -> int:
        return int(self.lib.jpxlg_ctx_cfl_fallbacks(self.handle))

    @property
    def cover_fallbacks(self) -> int:
        return int(self.lib.jpxlg_ctx_cover_fallbacks(self.handle))

    def stage_timing(self, enable: bool) -> None:
        self.check(self.lib.jpxlg_stage_timing(self.handle, int(enable)))

    def stage_times(self) -> dict:
        """Device milliseconds and kernel launches per stage since the last
        call (synchronizes)."""
        ms = np.zeros(len(STAGES), np.float64)
        ln = np.zeros(len(STAGES), np.uint64)
        n = self.lib.jpxlg_stage_times(self.handle, ms.ctypes.data, ln.ctypes.data, len(STAGES))
        if n < 0:
            self.check(n)
        return {name: (float(ms[i]), int(ln[i])) for i, name in enumerate(STAGES)}

    # -- encode ---------------------------------------------------------------
    def encode_transform(self, layout: "Layout", rgb: np.ndarray, req: EncodeRequest,
                         bits: int | None = None) -> Plan:
        rgb = np.ascontiguousarray(rgb)
        if bits is None:
            bits = 8 if rgb.dtype == np.uint8 else 16
        want = np.uint8 if bits == 8 else np.uint16
        if rgb.dtype != want or rgb.shape != (layout.height, layout.width, 3):
            raise ValueError(f"rgb must be {want.__name__} [{layout.height}, {layout.width}, 3]")
        plan = layout.empty_plan()
        s = plan._struct()
        p = req._struct()
        self.check(self.lib.jpxlg_encode_transform(self.handle, layout.handle,
                                                   rgb.ctypes.data, bits, C.byref(p),
                                                   C.byref(s), MEM_HOST))
        plan.lf_factors = (s.lf_factors[0], s.lf_factors[1])
        return plan

    def encode_stages(self, layout: "Layout", rgb: np.ndarray, req: EncodeRequest,
                      bits: int | None = None) -> dict:
        """Diagnostic: XYB, preconditioned planes and forward coefficients."""
        rgb = np.ascontiguousarray(rgb)
        if bits is None:
            bits = 8 if rgb.dtype == np.uint8 else 16
        h, w = layout.height, layout.width
        out = {"xyb": np.zeros((3, h, w), np.float32), "pre": np.zeros((3, h, w), np.float32),
               "coeff": np.zeros((3, 8 * layout.bh, 8 * layout.bw), np.float32)}
        p = req._struct()
        self.check(self.lib.jpxlg_encode_stages(self.handle, layout.handle, rgb.ctypes.data, bits,
                                                C.byref(p), out["xyb"].ctypes.data,
                                                out["pre"].ctypes.data, out["coeff"].ctypes.data))
        return out

    def probe(self, layout: "Layout", ref: "PrecomputedReference", rgb: np.ndarray,
              req: EncodeRequest, bits: int | None = None) -> float:
        """Encode, render at the source depth and score against ``ref``."""
        rgb = np.ascontiguousarray(rgb)
        if bits is None:
            bits = 8 if rgb.dtype == np.uint8 else 16
        out = C.c_double()
        p = req._struct()
        self.check(self.lib.jpxlg_probe(self.handle, layout.handle, ref.handle, rgb.ctypes.data,
                                        bits, C.byref(p), MEM_HOST, C.byref(out)))
        return out.value

    def probe_device(self, layout, ref, rgb_ptr: int, bits: int, req: EncodeRequest,
                     score_ptr: int) -> None:
        p = req._struct()
        self.check(self.lib.jpxlg_probe(self.handle, layout.handle, ref.handle,
                                        C.c_void_p(rgb_ptr), bits, C.byref(p), MEM_DEVICE,
                                        C.c_void_p(score_ptr)))


class Layout:
    """A validated cover and its per-block hf_mul / sharpness (jpxlg_layout)."""

    def __init__(self, ctx: Context, width: int, height: int, block_map: np.ndarray,
                 hf_mul: np.ndarray | int = 1, sharpness: np.ndarray | int | None = None):
        self.ctx = ctx
        self.width, self.height = width, height
        bw, bh = (width + 7) // 8, (height + 7) // 8
        self.block_map = np.ascontiguousarray(block_map, dtype=np.uint8).reshape(bh, bw)
        if np.isscalar(hf_mul):
            hf_mul = np.full((bh, bw), hf_mul, np.uint32)
        self.hf_mul = np.ascontiguousarray(hf_mul, dtype=np.uint32).reshape(bh, bw)
        if sharpness is None:
            sharpness = 0
        if np.isscalar(sharpness):
            sharpness = np.full((bh, bw), sharpness, np.uint8)
        self.sharpness = np.ascontiguousarray(sharpness, dtype=np.uint8).reshape(bh, bw)
        h = C.c_void_p()
        ctx.check(ctx.lib.jpxlg_layout_create(ctx.handle, width, height,
                                              self.block_map.ctypes.data,
                                              self.hf_mul.ctypes.data,
                                              self.sharpness.ctypes.data, C.byref(h)))
        self.handle = h
        self.bw, self.bh = bw, bh
        self.tw, self.th = (bw + 7) // 8, (bh + 7) // 8

    def empty_plan(self) -> Plan:
        return Plan(np.zeros((3, 8 * self.bh, 8 * self.bw), np.int32),
                    np.zeros((3, self.bh, self.bw), np.int32),
                    np.zeros((self.th, self.tw), np.int8),
                    np.zeros((self.th, self.tw), np.int8))

    def close(self):
        if self.handle:
            self.ctx.lib.jpxlg_layout_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PlanRenderer:
    """jpxl-plan-render lib.rs:560 PlanRenderer over the CUDA path."""

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def render(self, layout: Layout, plan: Plan, req: EncodeRequest, out: str = "srgb8",
               bits: int = 8) -> np.ndarray:
        kind = {"xyb": OUT_XYB, "linear": OUT_LINEAR, "srgb8": OUT_SRGB8,
                "linear_at_depth": OUT_LINEAR_DEPTH}[out]
        h, w = layout.height, layout.width
        res = (np.zeros((h, w, 3), np.uint8) if kind == OUT_SRGB8
               else np.zeros((3, h, w), np.float32))
        s = plan._struct()
        p = req._struct()
        self.ctx.check(self.ctx.lib.jpxlg_reconstruct(self.ctx.handle, layout.handle, C.byref(s),
                                                      C.byref(p), kind, bits, res.ctypes.data,
                                                      MEM_HOST))
        return res


class PrecomputedReference:
    """reference.rs:90 PrecomputedReference (Moments retention) on the device."""

    def __init__(self, ctx: Context, linear_rgb: np.ndarray | None = None, *,
                 device_ptr: int | None = None, width: int = 0, height: int = 0):
        self.ctx = ctx
        h = C.c_void_p()
        if device_ptr is not None:
            self.width, self.height = width, height
            rc = ctx.lib.jpxlg_ssim2_ref_create(ctx.handle, C.c_void_p(device_ptr), width,
                                                height, MEM_DEVICE, C.byref(h))
        else:
            planes = np.ascontiguousarray(linear_rgb, dtype=np.float32)
            if planes.ndim != 3 or planes.shape[0] != 3:
                raise ValueError("linear_rgb must be float32 [3, H, W]")
            self.height, self.width = planes.shape[1], planes.shape[2]
            rc = ctx.lib.jpxlg_ssim2_ref_create(ctx.handle, planes.ctypes.data, self.width,
                                                self.height, MEM_HOST, C.byref(h))
        ctx.check(rc)
        self.handle = h

    def close(self):
        if self.handle:
            self.ctx.lib.jpxlg_ssim2_ref_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Ssimulacra2Result:
    score: float
    raw_error: float
    terms: np.ndarray = field(default_factory=lambda: np.zeros(0))


class Ssimulacra2:
    """ssimulacra2.rs Ssimulacra2::score over the CUDA path."""

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def score(self, ref: PrecomputedReference, linear_rgb: np.ndarray) -> Ssimulacra2Result:
        planes = np.ascontiguousarray(linear_rgb, dtype=np.float32)
        if planes.shape != (3, ref.height, ref.width):
            raise JpxlError(-7, "candidate dimensions differ from the reference")
        sc, raw = C.c_double(), C.c_double()
        terms = np.zeros(6 * 18, np.float64)
        self.ctx.check(self.ctx.lib.jpxlg_ssim2_score(self.ctx.handle, ref.handle,
                                                      planes.ctypes.data, MEM_HOST,
                                                      C.byref(sc), C.byref(raw),
                                                      terms.ctypes.data))
        return Ssimulacra2Result(sc.value, raw.value, terms)

    def score_static_device(self, ref: PrecomputedReference, cand_ptr: int, out_ptr: int) -> None:
        """Queue an allocation-free score of device planes at `cand_ptr`
        ([3, H, W] float32) on the context's stream; `out_ptr` (device, 110
        float64) receives [score, raw error, terms...].  Frames up to
        2048 x 2048; calls in flight together on one device share scratch."""
        self.ctx.check(self.ctx.lib.jpxlg_ssim2_score_static(
            self.ctx.handle, ref.handle, C.c_void_p(cand_ptr), C.c_void_p(out_ptr)))


def select_blocks(ctx: Context, rgb: np.ndarray, req: EncodeRequest,
                  bits: int | None = None) -> np.ndarray:
    """The encoder's cover for a fixed quantizer (policy lib.rs:5260
    select_blocks): a uint8 [bh, bw] block map (DctSelect | ORIGIN on
    varblock origins) from interleaved RGB in host memory."""
    rgb = np.ascontiguousarray(rgb)
    if bits is None:
        bits = 8 if rgb.dtype == np.uint8 else 16
    h, w = rgb.shape[:2]
    out = np.zeros(((h + 7) // 8, (w + 7) // 8), np.uint8)
    p = req._struct()
    ctx.check(ctx.lib.jpxlg_select_blocks(ctx.handle, w, h, rgb.ctypes.data, bits, C.byref(p),
                                          out.ctypes.data, MEM_HOST))
    return out


def select_blocks_device(ctx: Context, width: int, height: int, rgb_ptr: int, bits: int,
                         req: EncodeRequest, map_ptr: int) -> None:
    """select_blocks on device RGB; the block map lands in device memory at
    map_ptr (ceil(w/8) * ceil(h/8) bytes), queued on the context's stream."""
    p = req._struct()
    ctx.check(ctx.lib.jpxlg_select_blocks(ctx.handle, width, height, C.c_void_p(rgb_ptr), bits,
                                          C.byref(p), C.c_void_p(map_ptr), MEM_DEVICE))


@dataclass
class BatchItem:
    """One probe of a batch: a frame (layout, reference, RGB in device memory)
    and a candidate's parameters."""

    layout: "Layout"
    ref: "PrecomputedReference"
    rgb_ptr: int
    bits: int
    req: EncodeRequest


class BatchProbe:
    """Many probes as one CUDA graph (jpxlg_batch_*): the quality controller's
    candidate sweep of quality.rs:2405 over evaluator.rs:295 probes."""

    def __init__(self, ctx: Context, items: list, lanes: int = 0):
        self.ctx = ctx
        self.items = list(items)
        arr = (BatchItemStruct * len(self.items))()
        for a, it in zip(arr, self.items):
            a.layout = it.layout.handle
            a.ref = it.ref.handle
            a.rgb = it.rgb_ptr
            a.bits = it.bits
            a.params = it.req._struct()
        self._arr = arr
        h = C.c_void_p()
        ctx.check(ctx.lib.jpxlg_batch_create(ctx.handle, len(self.items), arr, lanes,
                                             C.byref(h)))
        self.handle = h

    def run(self) -> np.ndarray:
        """Runs every probe; returns the scores in item order."""
        out = np.zeros(len(self.items), np.float64)
        self.ctx.check(self.ctx.lib.jpxlg_batch_run(self.ctx.handle, self.handle,
                                                    out.ctypes.data, MEM_HOST))
        return out

    def run_device(self, scores_ptr: int) -> None:
        """Queues every probe on the context's stream; scores land in the
        device array at scores_ptr (float64, one per item)."""
        self.ctx.check(self.ctx.lib.jpxlg_batch_run(self.ctx.handle, self.handle,
                                                    C.c_void_p(scores_ptr), MEM_DEVICE))

    def close(self):
        if getattr(self, "handle", None):
            self.ctx.lib.jpxlg_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SymbolDecoder:
    """jpxl-entropy decoder.rs SymbolDecoder over the library's host-side
    Annex C decoder (jpxlg_symbols_*): ``open`` reads the distribution bundle
    of an entropy-coded stream at bit ``bit_offset`` of ``data`` (LSB-first),
    ``read_uint`` pulls integers per context, ``finish`` checks the ANS final
    state.  Host code; no device is needed."""

    def __init__(self, data: bytes, num_dist: int, bit_offset: int = 0):
        self.lib = _lib.load()
        buf = np.frombuffer(bytes(data), np.uint8)
        h = C.c_void_p()
        rc = self.lib.jpxlg_symbols_open(buf.ctypes.data if buf.size else None, buf.size,
                                         bit_offset, num_dist, C.byref(h))
        if rc:
            raise JpxlError(rc, "jpxlg_symbols_open")
        self.handle = h

    def set_dist_multiplier(self, multiplier: int) -> None:
        self.lib.jpxlg_symbols_set_dist_multiplier(self.handle, multiplier)

    def read_uint(self, ctx: int) -> int:
        v = C.c_uint32()
        rc = self.lib.jpxlg_symbols_read(self.handle, ctx, C.byref(v))
        if rc:
            raise JpxlError(rc, f"jpxlg_symbols_read (context {ctx})")
        return v.value

    def read_many(self, contexts) -> np.ndarray:
        ctx = np.ascontiguousarray(contexts, np.uint32)
        out = np.zeros(ctx.size, np.uint32)
        rc = self.lib.jpxlg_symbols_read_many(self.handle, ctx.ctypes.data, ctx.size,
                                              out.ctypes.data)
        if rc:
            raise JpxlError(rc, "jpxlg_symbols_read_many")
        return out

    def finish(self) -> None:
        rc = self.lib.jpxlg_symbols_finish(self.handle)
        if rc:
            raise JpxlError(rc, "ANS stream did not end in its final state")

    @property
    def bits_read(self) -> int:
        return int(self.lib.jpxlg_symbols_bits_read(self.handle))

    def close(self):
        if self.handle:
            self.lib.jpxlg_symbols_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _CodestreamInfo(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("width", "height", "bits_per_sample", "xyb_encoded",
                                          "colour_space")] + [("transfer", C.c_int32)] + \
        [(n, C.c_uint32) for n in ("encoding", "num_passes", "gaborish", "gaborish_custom",
                                   "epf_iters", "x_qm_scale", "b_qm_scale",
                                   "adaptive_lf_smoothing", "global_scale", "quant_lf",
                                   "extra_precision", "default_matrices", "default_lf_dequant",
                                   "default_chroma_correlation")] + \
        [("x_factor_lf", C.c_int32), ("b_factor_lf", C.c_int32)] + \
        [(n, C.c_uint32) for n in ("blocks_w", "blocks_h", "num_varblocks", "num_channels",
                                   "sections", "sections_exact")] + \
        [("transform_counts", C.c_uint32 * 27)] + \
        [(n, C.c_uint32) for n in ("orientation", "num_extra")]


class CodestreamLimits(C.Structure):
    """jpxlg_codestream_limits (jpxl-core limits.rs Limits)."""

    _fields_ = [("max_pixels", C.c_uint64), ("max_alloc_bytes", C.c_uint64)]


class Codestream:
    """jpxl-decode's front end (decode.rs:400 decode up to the VarDCT
    frame's integer content, decode.rs:2513) over the library's host-side
    codestream reader (jpxlg_codestream_*).  ``info`` holds the headers'
    parameters; ``blocks()`` and ``coefficients()`` return the quantized LF,
    block map, HF multipliers, sharpness, CfL factors and coefficient image
    in the plan's layout.  Host code; no device is needed."""

    def __init__(self, data: bytes, max_pixels: int | None = None,
                 max_alloc_bytes: int | None = None):
        self.lib = _lib.load()
        buf = np.frombuffer(bytes(data), np.uint8)
        h = C.c_void_p()
        limits = None
        if max_pixels is not None or max_alloc_bytes is not None:
            # limits.rs Limits::new() defaults for the field not given
            limits = C.byref(CodestreamLimits(max_pixels or (1 << 30),
                                              max_alloc_bytes or (4 << 30)))
        rc = self.lib.jpxlg_codestream_open_limits(buf.ctypes.data if buf.size else None,
                                                   buf.size, limits, C.byref(h))
        if rc:
            raise JpxlError(rc, "jpxlg_codestream_open: " +
                            self.lib.jpxlg_codestream_last_error().decode())
        self.handle = h
        raw = _CodestreamInfo()
        self.lib.jpxlg_codestream_info(self.handle, C.byref(raw))
        self.info = {n: getattr(raw, n) for n, _ in _CodestreamInfo._fields_}
        self.info["transform_counts"] = list(raw.transform_counts)

    def blocks(self) -> dict:
        bw, bh = self.info["blocks_w"], self.info["blocks_h"]
        tw, th = (self.info["width"] + 63) // 64, (self.info["height"] + 63) // 64
        out = {"lf": np.zeros((3, bh, bw), np.int32), "block_map": np.zeros((bh, bw), np.uint8),
               "hf_mul": np.zeros((bh, bw), np.uint32), "sharpness": np.zeros((bh, bw), np.uint8),
               "cfl_x": np.zeros((th, tw), np.int8), "cfl_b": np.zeros((th, tw), np.int8)}
        rc = self.lib.jpxlg_codestream_blocks(self.handle, *(out[k].ctypes.data for k in (
            "lf", "block_map", "hf_mul", "sharpness", "cfl_x", "cfl_b")))
        if rc:
            raise JpxlError(rc, "jpxlg_codestream_blocks")
        return out

    def coefficients(self) -> np.ndarray:
        bw, bh = self.info["blocks_w"], self.info["blocks_h"]
        out = np.zeros((3, 8 * bh, 8 * bw), np.int32)
        rc = self.lib.jpxlg_codestream_coefficients(self.handle, out.ctypes.data)
        if rc:
            raise JpxlError(rc, "jpxlg_codestream_coefficients")
        return out

    def render(self, ctx: "Context", out: str = "srgb_float") -> np.ndarray:
        """The frame reconstructed on the GPU (jpxlg_codestream_render):
        float planes [3, H, W] for "xyb", "linear" and "srgb_float" (the
        decoder's unclipped float output), or [H, W, 3] uint8 for "srgb8".
        A grey image's samples are plane 0."""
        kinds = {"xyb": 0, "linear": 1, "srgb8": 2, "srgb_float": 4}
        w, h = self.info["width"], self.info["height"]
        buf = (np.zeros((h, w, 3), np.uint8) if out == "srgb8"
               else np.zeros((3, h, w), np.float32))
        ctx.check(self.lib.jpxlg_codestream_render(ctx.handle, self.handle, kinds[out],
                                                   buf.ctypes.data, MEM_HOST))
        return buf

    def extra(self, index: int) -> np.ndarray:
        """A frame's extra channel (alpha, ...) normalised to its bit depth,
        float32 [H, W]."""
        out = np.zeros((self.info["height"], self.info["width"]), np.float32)
        rc = self.lib.jpxlg_codestream_extra(self.handle, index, out.ctypes.data)
        if rc:
            raise JpxlError(rc, "jpxlg_codestream_extra")
        return out

    def channel(self, index: int) -> np.ndarray:
        out = np.zeros((self.info["height"], self.info["width"]), np.int32)
        rc = self.lib.jpxlg_codestream_channel(self.handle, index, out.ctypes.data)
        if rc:
            raise JpxlError(rc, "jpxlg_codestream_channel")
        return out

    def close(self):
        if getattr(self, "handle", None):
            self.lib.jpxlg_codestream_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def open_codestreams(datas, workers: int | None = None, max_pixels: int | None = None,
                     max_alloc_bytes: int | None = None) -> list:
    """Codestream(d) for every d in datas, in order, parsed on up to
    `workers` host threads (default: one per core).  The reader keeps its
    allocation meter and last error per thread and ctypes releases the GIL
    around it, so independent streams parse in parallel.  If any stream is
    rejected, the others are closed and its JpxlError is raised."""
    import os
    from concurrent.futures import ThreadPoolExecutor

    datas = list(datas)
    n = workers if workers is not None else (os.cpu_count() or 1)
    n = max(1, min(n, len(datas)))

    def open_one(d):
        return Codestream(d, max_pixels=max_pixels, max_alloc_bytes=max_alloc_bytes)

    if n == 1:
        opened = []
        try:
            for d in datas:
                opened.append(open_one(d))
        except Exception:
            for s in opened:
                s.close()
            raise
        return opened
    with ThreadPoolExecutor(n) as ex:
        futures = [ex.submit(open_one, d) for d in datas]
    opened, error = [], None
    for f in futures:
        try:
            opened.append(f.result())
        except Exception as e:  # noqa: BLE001 - re-raised below
            error = error or e
    if error is not None:
        for s in opened:
            s.close()
        raise error
    return opened


class DecodeBatch:
    """Many opened streams rendered by one graph launch (jpxlg_decode_batch_*):
    a loop of decode.rs:400 decode calls as one CUDA graph.  The streams must
    stay open while the batch lives."""

    KINDS = {"xyb": 0, "linear": 1, "srgb8": 2, "srgb_float": 4}

    def __init__(self, ctx: Context, streams: list, out: str = "srgb8", lanes: int = 0,
                 precision: str = "fp32"):
        self.ctx, self.streams, self.out = ctx, list(streams), out
        arr = (C.c_void_p * len(self.streams))(*[s.handle.value for s in self.streams])
        h = C.c_void_p()
        ctx.check(ctx.lib.jpxlg_decode_batch_create(ctx.handle, len(self.streams), arr,
                                                    self.KINDS[out], PRECISIONS[precision],
                                                    lanes, C.byref(h)))
        self.handle = h
        self.buffers = []
        for s in self.streams:
            w, hh = s.info["width"], s.info["height"]
            self.buffers.append(np.zeros((hh, w, 3), np.uint8) if out == "srgb8"
                                else np.zeros((3, hh, w), np.float32))
        self._outs = (C.c_void_p * len(self.buffers))(*[b.ctypes.data for b in self.buffers])

    def run(self, copy: bool = True) -> list:
        """Launches the graph and waits; returns every stream's pixels (the
        same arrays each run) unless copy is False."""
        self.ctx.check(self.ctx.lib.jpxlg_decode_batch_run(
            self.ctx.handle, self.handle, self._outs if copy else None, MEM_HOST))
        return self.buffers

    def close(self):
        if getattr(self, "handle", None):
            self.ctx.lib.jpxlg_decode_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


SPECIAL_KINDS = {"dct2x2": 1, "hornuss": 2, "dct4x4": 3, "dct8x4": 4, "dct4x8": 5,
                 "afv0": 6, "afv1": 7, "afv2": 8, "afv3": 9}


def special_blocks(ctx: Context, kind: int, coef: np.ndarray) -> np.ndarray:
    """The decoder's 8x8 special transforms (varblock.rs:1218) on dequantized
    coefficient blocks, float32 [n, 8, 8] (LLF at [0, 0]) -> samples
    [n, 8, 8], through the kernels the stream render uses."""
    c = np.ascontiguousarray(coef, np.float32).reshape(-1, 64)
    out = np.zeros_like(c)
    ctx.check(ctx.lib.jpxlg_diag_special_blocks(ctx.handle, kind, c.ctypes.data, c.shape[0],
                                                out.ctypes.data, MEM_HOST))
    return out.reshape(-1, 8, 8)


def score_pair(ctx: Context, ref_rgb: np.ndarray, cand_rgb: np.ndarray) -> float:
    """jpxl-perceptual lib.rs:195 score_pair on linear [3, H, W] planes."""
    a = np.ascontiguousarray(ref_rgb, dtype=np.float32)
    b = np.ascontiguousarray(cand_rgb, dtype=np.float32)
    if a.shape != b.shape:
        raise JpxlError(-7, "dimension mismatch")
    out = C.c_double()
    ctx.check(ctx.lib.jpxlg_score_pair(ctx.handle, a.ctypes.data, b.ctypes.data, a.shape[2],
                                       a.shape[1], MEM_HOST, C.byref(out)))
    return out.value


def srgb_to_linear_planes(rgb: np.ndarray, bits: int = 8) -> np.ndarray:
    """Source code points -> linear planes through the reference's per-code-point
    curve (source.rs:226/:355, evaluator.rs:88), as float32 [3, H, W]."""
    maxv = 255.0 if bits == 8 else float(min(65535, (1 << bits) - 1))
    lut = np.empty(256 if bits == 8 else 65536, np.float32)
    v = (np.arange(lut.size, dtype=np.float32) / np.float32(maxv)).astype(np.float32)
    a = np.abs(v)
    lin = np.where(a <= np.float32(12.92) * np.float32(0.0031308), a / np.float32(12.92),
                   np.power((a + np.float32(0.055)) / np.float32(1.055), np.float32(2.4)))
    lut[:] = lin.astype(np.float32)
    return np.ascontiguousarray(lut[rgb].transpose(2, 0, 1))
