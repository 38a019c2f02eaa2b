"""Writes dim5_vectors.json: the ten 4-body events and their five variables that the reference's
Dim5 known-answer test holds (tests/simple/VectorsTest.cu:10-36), read from that file as text.

Run with the path of a GooFit source tree, as an argument or in $GOOFIT_REFERENCE:
    python tests/golden/make_dim5_vectors.py <path-to-GooFit>
Each event row is 16 numbers, (px, py, pz, E) of the daughters 0..3; each answer row is
(m12, m34, cos12, cos34, phi); the test's tolerance is Approx(...).epsilon(1e-5).
"""
import json
import os
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def numbers_after(text: str, name: str) -> list[float]:
    body = text.split(f"{name} <<", 1)[1].split(";", 1)[0]
    return [float(x) for x in re.findall(r"-?\d+\.?\d*(?:e-?\d+)?", body)]


def main() -> None:
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GOOFIT_REFERENCE")
    if not src:
        sys.exit("usage: make_dim5_vectors.py <path-to-GooFit> (or set GOOFIT_REFERENCE)")
    text = (Path(src) / "tests" / "simple" / "VectorsTest.cu").read_text()
    m = numbers_after(text, "matI")
    f = numbers_after(text, "finalsI")
    assert len(m) == 160 and len(f) == 50, (len(m), len(f))
    out = {"source": "tests/simple/VectorsTest.cu:10-36", "epsilon": 1e-5,
           "events": [m[16 * i:16 * i + 16] for i in range(10)],
           "answers": [f[5 * i:5 * i + 5] for i in range(10)]}
    (HERE / "dim5_vectors.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
