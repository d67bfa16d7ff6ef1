"""Regenerate spectral_tables.npz from the reference checkout.

The spectral upsampling must reproduce the reference's numbers exactly, so the
renderer needs the same data the reference bakes into its headers:
  * CIE 1931 2-degree colour-matching functions, 360-780 nm at 1 nm
    (core/spectrum/ciexyz.cuh:86-520) and the CIE D65 illuminant SPD
    (core/spectrum/ciexyz.cuh:11-65) -- public CIE standard data;
  * the trained weights of the two residual MLPs that map RGB and wavelength
    to a 4-term spectral basis (core/spectrum/spectrum_basis.cuh:16-2259).
Only numeric tables are extracted; the code that uses them is our own
(aperturerendererv3_gb300/csrc/ar_spectral.h).  Run from the repository root:

    python aperturerendererv3_gb300/data/make_spectral_tables.py [reference_root]
"""
from __future__ import annotations

import re
import os
import sys
from pathlib import Path

import numpy as np

NUM = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?")

RGB_LAYERS = ["RGB_IN_W", "RGB_IN_B"] + [f"RGB_BLK{i}_{k}" for i in range(7) for k in "WB"] + ["RGB_OUT_W"]
LAM_LAYERS = [f"LAM_BLK{i}_{k}" for i in range(7) for k in "WB"] + ["LAM_OUT_W"]


def _array(text: str, name: str, count: int) -> np.ndarray:
    # the last declaration of NAME[...] is followed by the initializer
    decl = [m.end() for m in re.finditer(r"\b" + re.escape(name) + r"\s*\[[^\]]*\]\s*=", text)]
    if not decl:
        raise KeyError(name)
    start = text.index("{", decl[-1])
    end = text.index("};", start)
    body = text[start + 1:end].replace("float3", " ")
    vals = np.array([float(v) for v in NUM.findall(body)], dtype=np.float32)
    if vals.size != count:
        raise ValueError(f"{name}: expected {count} values, got {vals.size}")
    return vals


def extract(ref_root: Path) -> dict[str, np.ndarray]:
    cie = (ref_root / "core/spectrum/ciexyz.cuh").read_text()
    basis = (ref_root / "core/spectrum/spectrum_basis.cuh").read_text()
    out = {
        "D65_SPD": _array(cie, "D65_SPD", 421),
        "CIEXYZ_CMF": _array(cie, "CIEXYZ_CMF", 421 * 3).reshape(421, 3),
    }
    sizes = {"IN_W": 32 * 32, "IN_B": 32, "OUT_W": 4 * 32}
    for name in RGB_LAYERS + LAM_LAYERS:
        suffix = name.split("_", 1)[1]
        n = sizes.get(suffix, 32 * 32 if suffix.endswith("_W") else 32)
        out[name] = _array(basis, name, n)
    return out


def main() -> None:
    if len(sys.argv) > 1:
        ref_root = Path(sys.argv[1])
    elif os.environ.get("AR_REFERENCE_ROOT"):
        ref_root = Path(os.environ["AR_REFERENCE_ROOT"])
    else:
        sys.exit("usage: make_spectral_tables.py REFERENCE_CHECKOUT (or set AR_REFERENCE_ROOT)")
    tables = extract(ref_root)
    dst = Path(__file__).resolve().parent / "spectral_tables.npz"
    np.savez(dst, **tables)
    print("wrote", dst, {k: v.shape for k, v in tables.items()})


if __name__ == "__main__":
    main()
