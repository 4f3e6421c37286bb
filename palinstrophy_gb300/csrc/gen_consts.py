"""Write pal_consts.h: cos/sin(2 pi e / R) for the in-register DFT sizes.

The values are evaluated with mpmath at 40 digits and printed with 25
significant digits, so the compiler rounds each literal to the nearest double
(and, through the double, to float).  Run from this directory:

    python gen_consts.py > pal_consts.h
"""
import mpmath

mpmath.mp.dps = 40
SIZES = (6, 8, 12, 16, 24, 32, 48, 64)

print("// Generated by gen_consts.py -- exact cos/sin(2*pi*e/R) literals.")
print("#pragma once")
print("namespace pal {")
print("template <int R> struct Trig;")
for R in SIZES:
    cs = [mpmath.cos(2 * mpmath.pi * e / R) for e in range(R)]
    sn = [mpmath.sin(2 * mpmath.pi * e / R) for e in range(R)]
    fmt = lambda v: mpmath.nstr(v, 25, min_fixed=-5, max_fixed=5) if abs(v) > 1e-30 else "0.0"
    print(f"template <> struct Trig<{R}> {{")
    print("  static constexpr double c[%d] = {%s};" % (R, ", ".join(fmt(v) for v in cs)))
    print("  static constexpr double s[%d] = {%s};" % (R, ", ".join(fmt(v) for v in sn)))
    print("};")
print("}  // namespace pal")
