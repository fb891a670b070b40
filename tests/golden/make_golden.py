"""Extracts the reference's constant tables and recorded known answers into
tests/golden/reference_constants.json.

Run in a checkout that has the reference source at /root/reference (it is
not present where the tests run; the JSON is the committed fixture):

    python tests/golden/make_golden.py

Sources (JPXL/crates/...):
  jpxl-core/src/dct.rs:148-211          DCT4_4 / DCT4_8 / DCT4_16 leaf matrices
  jpxl-perceptual/src/ssimulacra2.rs:391 WEIGHTS
  jpxl-core/src/dequant.rs:712-1020      Table I.6 DCT parameter rows
  jpxl-perceptual/src/blur.rs:41/:47     MUL_IN / MUL_PREV
  jpxl-core/src/varblock.rs AFV_BASIS    Table I.11, the AFV basis
  .akr/records/jpegxl-rs/evidence.akr:6424  recorded score bits of the 4.3 MP pair
"""
from __future__ import annotations

import json
import re
from pathlib import Path

REF = Path("/root/reference/JPXL/crates")
OUT = Path(__file__).resolve().parent / "reference_constants.json"

NUM = r"-?\d[\d_]*\.?[\d_]*(?:e-?\d+)?"


def numbers(text: str) -> list[float]:
    return [float(x.replace("_", "")) for x in re.findall(NUM, text)]


def block(src: str, name: str) -> str:
    m = re.search(r"const " + name + r"\b[^=]*=\s*\[(.*?)\];\n", src, re.S)
    if not m:
        raise KeyError(name)
    return m.group(1)


def main() -> None:
    dct = (REF / "jpxl-core/src/dct.rs").read_text()
    out: dict = {}
    for name in ("DCT4_4", "DCT4_8", "DCT4_16"):
        out[name] = numbers(block(dct, name))
    ss = (REF / "jpxl-perceptual/src/ssimulacra2.rs").read_text()
    out["SSIM_WEIGHTS"] = numbers(block(ss, "WEIGHTS"))
    blur = (REF / "jpxl-perceptual/src/blur.rs").read_text()
    out["MUL_IN"] = numbers(block(blur, "MUL_IN"))
    out["MUL_PREV"] = numbers(block(blur, "MUL_PREV"))
    dq = (REF / "jpxl-core/src/dequant.rs").read_text()
    for name in ("DCT8X8_PARAMS", "DCT16X16_PARAMS", "DCT32X32_PARAMS", "DCT16X8_PARAMS",
                 "DCT32X8_PARAMS", "DCT16X32_PARAMS"):
        vals = numbers(block(dq, name))
        n = len(vals) // 3
        out[name] = [vals[i * n:(i + 1) * n] for i in range(3)]
    vb = (REF / "jpxl-core/src/varblock.rs").read_text()
    afv = numbers(block(vb, "AFV_BASIS"))
    if len(afv) != 256:
        raise ValueError(f"AFV_BASIS: {len(afv)} entries")
    out["AFV_BASIS"] = [afv[i * 16:(i + 1) * 16] for i in range(16)]
    ev = Path("/root/reference/.akr/records/jpegxl-rs/evidence.akr").read_text()
    m = re.search(r"Raw score bits ([0-9a-f]{16})", ev)
    out["SCORE_BITS_4MP_PAIR"] = m.group(1) if m else None
    # Hand-derived known answers printed in the reference's own tests.
    out["KAT"] = {
        "dct_ii_8_constant_dc": 2.828427,          # dct.rs:1572
        "dct_ii_8_impulse": [0.35355339, 0.49039264],
        "gaborish_impulse_w1_0.25_w2_0.125": [[0.05, 0.1, 0.05], [0.1, 0.4, 0.1],
                                              [0.05, 0.1, 0.05]],  # decode gaborish.rs:748
        "epf_step2_three_pixel_row": 0.720751,     # decode epf.rs:1186
        "epf_step2_tap_weight": 0.5811627,
        "hf_multiplier_32768_2": 1.0,              # reconstruct.rs:122
        "bias_adjust_10_0.9_0.145": 9.9855,
        "positive_xyb_black": [0.42, 0.01, 0.55],  # perceptual color.rs tests
        "identical_256x192_score": 100.0,          # perceptual tests/metric.rs:20
    }
    OUT.write_text(json.dumps(out, indent=1))
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
