"""Writes ar_t_quantile.h: the upper 0.25 % quantiles of Student's t
distribution for 1..1024 degrees of freedom (the two-sided 0.5 % critical
values of a t-test), rounded to float.  These are the values the reference's
denoiser looks its Welch t-test thresholds up in (core/denoise/t_quantile.cu,
T005QuantilesHost / T005QuantilesDev, indexed by floor(nu) - 1).

Run from this directory: python gen_t_quantile.py  (needs scipy)."""
from pathlib import Path

import numpy as np
from scipy import stats

SIZE = 1024
ALPHA_TWO_SIDED = 0.005


def table() -> np.ndarray:
    nu = np.arange(1, SIZE + 1, dtype=np.float64)
    return stats.t.ppf(1.0 - ALPHA_TWO_SIDED / 2.0, nu).astype(np.float32)


def main() -> None:
    t = table()
    rows = []
    for i in range(0, SIZE, 4):
        rows.append("    " + ", ".join(f"{float(v).hex()}f" for v in t[i:i + 4]) + ",")
    text = ("// Generated by gen_t_quantile.py: Student t quantiles at 1 - 0.0025 for\n"
            "// nu = 1..1024 (float).  Do not edit.\n#pragma once\n\n"
            f"#define AR_T_QUANTILE_COUNT {SIZE}\n"
            "static const float ar_t_quantile_0025[AR_T_QUANTILE_COUNT] = {\n" + "\n".join(rows) + "\n};\n")
    Path(__file__).with_name("ar_t_quantile.h").write_text(text)


if __name__ == "__main__":
    main()
