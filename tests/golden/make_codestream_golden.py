"""Copies the reference's cjxl-encoded VarDCT fixtures and their djxl
decodes into tests/golden/codestream/ (the .jxl codestreams and .npy pixel
references are test data; nothing of the reference's source is copied).

Run in a checkout that has the reference source at /root/reference (it is
not present where the tests run; the copied files are the committed fixture):

    python tests/golden/make_codestream_golden.py

Source: JPXL/tests/fixtures/handmade/{03..07,09,11,12,14..16,21,40,50..53,60,63,64,70..73,80..84,100..107,109,110}_*.jxl with the .npy decodes
committed beside them (djxl v0.13.0 196a43d9 --output_format npy; provenance
in each fixture's .jxl.txt sidecar; 64 and the lossless fixtures have none).
110 (photon noise) is the stream the reader reports as unsupported.
"""
from __future__ import annotations

import shutil
from pathlib import Path

SRC = Path("/root/reference/JPXL/tests/fixtures/handmade")
OUT = Path(__file__).resolve().parent / "codestream"
NAMES = ["03_gradient_8x8_lossless",
         "04_gradient_8x8_lossy",
         "11_modular_gradient_256x256_lossless",
         "40_checker_64x64_lossless",
         "60_sawtooth_32x32_lossless",
         "72_lfframe_gray_128x128_nofilters",
         "73_progressive_all_gray_128x128_nofilters",
         "82_alpha_vardct_rgba_64x64_nofilters",
         "83_alpha_vardct_rgba_384x320_nofilters",
         "84_alpha_vardct_ga_128x128_nofilters",
         "110_noise_rgb_32x32",
         "80_alpha_rgba_8x8_lossless",
         "81_alpha_rgba_600x520_lossless",
         "05_gradient_300x200_lossless",
         "12_modular_gray_300x200_lossless",
         "21_gradient_260x10_lossless",
         "14_modular_gray_600x520_multisection_lossless",
         "15_modular_rgb_600x520_multisection_lossless",
         "16_modular_gray_511x8_multisection_lossless",
         "100_orientation_identity_rgba_24x16",
         "101_orientation_flip_h_rgba_24x16",
         "102_orientation_rot180_rgba_24x16",
         "103_orientation_flip_v_rgba_24x16",
         "104_orientation_transpose_rgba_24x16",
         "105_orientation_rot90cw_rgba_24x16",
         "106_orientation_antitranspose_rgba_24x16",
         "107_orientation_rot90ccw_rgba_24x16",
         "109_orientation_transpose_vardct_rgba_64x64",
         "06_gradient_300x200_lossy",
         "07_modular_gray_8x8_lossless",
         "09_modular_rgb_64x64_lossless",
         "50_vardct_mixed_gray_128x128_nofilters_d1",
         "51_vardct_mixed_gray_128x128_nofilters_d4",
         "52_vardct_mixed_gray_128x128_filters_d1",
         "53_vardct_mixed_gray_128x128_filters_d4",
         "63_vardct_outofgamut_rgb_64x64_nofilters_d4",
         "64_vardct_lfgroupseam_rgb_128x2176_nofilters_d6",
         "70_progressive_ac_gray_128x128_nofilters",
         "71_qprogressive_ac_gray_128x128_nofilters"]


def main() -> None:
    OUT.mkdir(exist_ok=True)
    for name in NAMES:
        for ext in (".jxl", ".npy"):
            src = SRC / (name + ext)
            if src.exists():
                shutil.copyfile(src, OUT / src.name)
                print("copied", src.name)


if __name__ == "__main__":
    main()
