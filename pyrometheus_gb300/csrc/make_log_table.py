"""Writes log_table.cuh for the table-driven logarithm of pyro_math.cuh:
for F_j = 1 + j/128, j = 0..128, the correctly rounded 1/F_j and ln F_j
split as hi + lo (hi = ln F_j rounded to double, lo = the rounded rest),
plus ln 2 split so that m * LN2_HI is exact for |m| < 2^11, and 1/ln 10
(60-digit mpmath evaluation).

    python pyrometheus_gb300/csrc/make_log_table.py
"""

import os

import mpmath

N = 128
mpmath.mp.dps = 60


def rn(x) -> float:
    return float(mpmath.mpf(x))


def main():
    rows = []
    for j in range(N + 1):
        F = 1 + mpmath.mpf(j) / N
        inv = rn(1 / F)
        lf = mpmath.log(F)
        hi = rn(lf)
        lo = rn(lf - mpmath.mpf(hi))
        rows.append((inv, hi, lo))
    ln2 = mpmath.log(2)
    e = int(mpmath.floor(mpmath.log(ln2, 2)))
    scale = mpmath.mpf(2) ** (41 - e)      # 42 significant bits
    ln2_hi = rn(mpmath.floor(ln2 * scale) / scale)
    ln2_lo = rn(ln2 - mpmath.mpf(ln2_hi))
    inv_ln10 = rn(1 / mpmath.log(10))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                       "log_table.cuh")
    with open(out, "w") as f:
        f.write("// Generated by make_log_table.py: for F = 1 + j/128, "
                "j = 0..128,\n// {1/F, ln F (hi), ln F - hi (lo)} correctly "
                "rounded.\n#pragma once\n\n")
        f.write(f"#define PYRO_LOG_N {N}\n")
        f.write(f"#define PYRO_LOG_LN2_HI {float.hex(ln2_hi)}  "
                "// ln 2, 42 bits\n")
        f.write(f"#define PYRO_LOG_LN2_LO {float.hex(ln2_lo)}  "
                "// ln 2 - hi\n")
        f.write(f"#define PYRO_LOG_INV_LN10 {float.hex(inv_ln10)}\n\n")
        f.write("__device__ const double pyro_log_table[3 * (PYRO_LOG_N + 1)]"
                " = {\n")
        for inv, hi, lo in rows:
            f.write(f"    {float.hex(inv)}, {float.hex(hi)}, "
                    f"{float.hex(lo)},\n")
        f.write("};\n")


if __name__ == "__main__":
    main()
