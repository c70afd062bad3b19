"""Generates the constant tables of the project sin/cos (float-float values of sin and cos at
j*pi/256, j = 0..511, and the float split of pi/256) from 300-bit mpmath evaluations. The same table
is written for the CUDA sources (b2g_trig_table.h) and for the CPU oracle (oracle/trig_table.h);
a test checks the two are identical and exact.

    python box2dpp_gb300/csrc/gen_trig_table.py
"""
import os

import mpmath
import numpy as np

mpmath.mp.prec = 300
HERE = os.path.dirname(os.path.abspath(__file__))


def f32(x) -> np.float32:
    """Round a high-precision value to the nearest float32 (ties to even) via exact double steps."""
    d = float(x)  # nearest double
    f = np.float32(d)
    # correct a possible double rounding: compare against the exact value
    below = np.nextafter(f, np.float32(-np.inf))
    above = np.nextafter(f, np.float32(np.inf))
    best = min((f, below, above), key=lambda c: (abs(mpmath.mpf(float(c)) - x), int(np.frombuffer(c.tobytes(), np.uint32)[0]) & 1))
    return np.float32(best)


def hexf(v: np.float32) -> str:
    return float(v).hex() + "f"


def tables():
    step = mpmath.pi / 256
    rows = []
    for j in range(512):
        s, c = mpmath.sin(j * step), mpmath.cos(j * step)
        sh = f32(s); sl = f32(s - mpmath.mpf(float(sh)))
        ch = f32(c); cl = f32(c - mpmath.mpf(float(ch)))
        rows.append((sh, sl, ch, cl))
    c1 = f32(step); c2 = f32(step - mpmath.mpf(float(c1)))
    c3 = f32(step - mpmath.mpf(float(c1)) - mpmath.mpf(float(c2)))
    inv = f32(256 / mpmath.pi)
    return rows, (c1, c2, c3, inv)


def write(path: str, prefix: str, guard: str):
    rows, (c1, c2, c3, inv) = tables()
    with open(path, "w") as f:
        f.write("// Generated by box2dpp_gb300/csrc/gen_trig_table.py: float-float sin and cos of j*pi/256\n")
        f.write("// (j = 0..511) and the float split of pi/256. Do not edit.\n")
        f.write(f"#ifndef {guard}\n#define {guard}\n")
        f.write(f"#define {prefix}PIO256_1 {hexf(c1)}\n#define {prefix}PIO256_2 {hexf(c2)}\n")
        f.write(f"#define {prefix}PIO256_3 {hexf(c3)}\n#define {prefix}INV_PIO256 {hexf(inv)}\n")
        f.write(f"#define {prefix}TRIG_TABLE_ROWS \\\n")
        for j, (sh, sl, ch, cl) in enumerate(rows):
            end = ", \\\n" if j < 511 else "\n"
            f.write(f"    {hexf(sh)}, {hexf(sl)}, {hexf(ch)}, {hexf(cl)}{end}")
        f.write("#endif\n")


if __name__ == "__main__":
    write(os.path.join(HERE, "b2g_trig_table.h"), "B2G_", "B2G_TRIG_TABLE_H")
    write(os.path.join(HERE, "..", "..", "oracle", "trig_table.h"), "B2O_", "B2O_TRIG_TABLE_H")
    print("ok")
