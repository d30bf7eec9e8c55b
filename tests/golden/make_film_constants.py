"""Extracts the film path's colour constants from the reference tree as text.

Reads core/spectrum.h of the StatER tree (pbrt-v3's XYZToRGB, RGBToXYZ and
RGBSpectrum::y), parses the float literals of each function body and stores them
with the lines they came from in film_constants.json next to this script. The
oracle's film restatement is checked against that fixture, which pins the
constants of Film::UpdateImage's XYZ round trip and of the luminance clamp.

Needs the reference tree, named by STATER_REFERENCE; run from the repository root:
    STATER_REFERENCE=<StatER tree> python tests/golden/make_film_constants.py
"""
from __future__ import annotations

import json
import os
import re
from pathlib import Path

OUT = Path(__file__).resolve().parent / "film_constants.json"
REF = Path(os.environ.get("STATER_REFERENCE", ""))


def body(lines, signature):
    """(first line number, text) of the brace-delimited body after `signature`."""
    for i, line in enumerate(lines):
        if signature in line:
            depth, out = 0, []
            for j in range(i, len(lines)):
                out.append(lines[j])
                depth += lines[j].count("{") - lines[j].count("}")
                if depth == 0 and "}" in lines[j]:
                    return i + 1, j + 1, "".join(out)
    raise KeyError(signature)


def literals(text):
    # the sign binds to the literal: "a - 1.5f * x" contributes -1.5
    vals = []
    for m in re.finditer(r"([-+])?\s*(\d+\.\d+)f", text):
        v = float(m.group(2))
        vals.append(-v if m.group(1) == "-" else v)
    return vals


def main():
    if not str(REF) or not (REF / "src" / "core" / "spectrum.h").exists():
        raise SystemExit("set STATER_REFERENCE to the StatER tree (src/core/spectrum.h not found)")
    src = REF / "src" / "core" / "spectrum.h"
    lines = src.read_text().splitlines(keepends=True)
    out = {"source": "src/core/spectrum.h"}
    for name, sig in [("xyz_to_rgb", "inline void XYZToRGB(const Float xyz[3], Float rgb[3])"),
                      ("rgb_to_xyz", "inline void RGBToXYZ(const Float rgb[3], Float xyz[3])")]:
        a, b, text = body(lines, sig)
        vals = literals(text)
        assert len(vals) == 9, (name, vals)
        out[name] = [vals[0:3], vals[3:6], vals[6:9]]
        out[name + "_lines"] = f"{a}-{b}"
    # RGBSpectrum::y(): the second y() in the header (the first is SampledSpectrum's)
    idx = [i for i, l in enumerate(lines) if "const Float YWeight[3]" in l]
    assert len(idx) == 1
    out["y_weight"] = literals(lines[idx[0]])
    out["y_weight_lines"] = f"{idx[0] + 1}"
    assert len(out["y_weight"]) == 3
    OUT.write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
