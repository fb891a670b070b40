"""Copies the reference's entropy-coded fixtures into
tests/golden/entropy_vectors.json: each carved payload (bytes, re-packed
LSB-first from the stream's first bit), the number of pre-clustered contexts,
the context of each read and the integers the stream decodes to.

Run in a checkout that has the reference source at /root/reference (it is
not present where the tests run; the JSON is the committed fixture):

    python tests/golden/make_entropy_golden.py

Source: JPXL/crates/jpxl-entropy/tests/fixtures/entropy/*.bin with their
.expected and .bin.txt sidecars (carved from cjxl-produced files by the
reference's authors; 07_ma_tree is the MA-tree stream of
tests/fixtures/handmade/07_modular_gray_8x8_lossless.jxl).
"""
from __future__ import annotations

import json
from pathlib import Path

SRC = Path("/root/reference/JPXL/crates/jpxl-entropy/tests/fixtures/entropy")
OUT = Path(__file__).resolve().parent / "entropy_vectors.json"


def main() -> None:
    vectors = []
    for binf in sorted(SRC.glob("*.bin")):
        lines = [ln.split() for ln in binf.with_suffix(".expected").read_text().splitlines()
                 if ln.strip() and not ln.startswith("#")]
        num_dist = int(lines[0][0])
        contexts = [int(x) for x in lines[1]]
        expected = [int(x) for x in lines[2]]
        assert len(contexts) == len(expected)
        provenance = binf.with_name(binf.name + ".txt").read_text().splitlines()[:3]
        vectors.append({"name": binf.stem, "payload_hex": binf.read_bytes().hex(),
                        "num_dist": num_dist, "contexts": contexts, "expected": expected,
                        "provenance": " ".join(x.strip() for x in provenance)})
    OUT.write_text(json.dumps({"vectors": vectors}, indent=1) + "\n")
    print(f"wrote {len(vectors)} vectors to {OUT}")


if __name__ == "__main__":
    main()
