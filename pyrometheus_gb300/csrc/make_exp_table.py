"""Writes exp_table.cuh: 2^(j/2048), j = 0..2047, correctly rounded to
double (60-digit mpmath evaluation), plus ln2/2048 rounded to double and
its Cody-Waite split, for the table-driven exponential of pyro_math.cuh.

    python pyrometheus_gb300/csrc/make_exp_table.py
"""

import os

import mpmath

N = 2048
mpmath.mp.dps = 60


def rn(x) -> float:
    """Round an mpmath value to the nearest double."""
    return float(mpmath.mpf(x))


def main():
    vals = [rn(mpmath.power(2, mpmath.mpf(j) / N)) for j in range(N)]
    ln2_n = mpmath.log(2) / N
    # leading part with 32 significant bits so kd * L1 is exact for
    # |kd| < 2^21 (|x| < 708 gives |kd| < 2.1e6 < 2^21)
    e = int(mpmath.floor(mpmath.log(ln2_n, 2)))
    scale = mpmath.mpf(2) ** (31 - e)
    l1 = rn(mpmath.floor(ln2_n * scale) / scale)
    l2 = rn(ln2_n - mpmath.mpf(l1))
    inv = rn(N / mpmath.log(2))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                       "exp_table.cuh")
    with open(out, "w") as f:
        f.write("// Generated by make_exp_table.py: 2^(j/2048) correctly "
                "rounded, j = 0..2047.\n#pragma once\n\n")
        f.write(f"#define PYRO_EXP_N {N}\n")
        f.write(f"#define PYRO_EXP_INV_L {float.hex(inv)}  // 2048/ln2\n")
        f.write(f"#define PYRO_EXP_L {float.hex(rn(ln2_n))}  // ln2/2048\n")
        f.write(f"#define PYRO_EXP_L1 {float.hex(l1)}  // ln2/2048, 32 bits\n")
        f.write(f"#define PYRO_EXP_L2 {float.hex(l2)}  // ln2/2048 - L1\n\n")
        f.write("__device__ const double pyro_exp_table[PYRO_EXP_N] = {\n")
        for i in range(0, N, 4):
            f.write("    " + ", ".join(float.hex(v) for v in vals[i:i + 4])
                    + ",\n")
        f.write("};\n")


if __name__ == "__main__":
    main()
