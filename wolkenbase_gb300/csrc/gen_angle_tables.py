"""Writes angle_tables.h: the integer-angle tables used by atan2i.

wolkenbase fills three tables at start-up (angle.cpp:305-320) with
long-double tan/sin/cos of the angles i*2^20 - 0xff00000 (tan, 511 entries)
and i*2^20 - 0xff80000 (sin, cos, 512 entries), an angle unit being
2^-31 turn; BoundRect::include (boundrect.cpp:44-58) evaluates sin/cos of the
four quadrant angles the same way.  The long double is the x86-64 80-bit
format: the argument is (angle * pi_64) rounded to a 64-bit significand,
divided by 2^30; the function value is rounded to 64 bits and then to double.

This script recomputes those values with mpmath at 200 bits and performs the
same two roundings, so the GPU library carries fixed tables that do not
depend on the host's long double.  The same script also writes the
double-double of 0x40000000/M_PIl used by atan2i's final correction step.
Run: python gen_angle_tables.py > angle_tables.h
"""
import sys

import mpmath as mp

mp.mp.prec = 200


def round_bits(x, bits):
    if x == 0:
        return mp.mpf(0)
    m, e = mp.frexp(x)
    return mp.ldexp(mp.nint(mp.ldexp(m, bits)), e - bits)


PI64 = round_bits(mp.pi, 64)


def x87(fn, angle):
    arg = round_bits(mp.mpf(angle) * PI64, 64) / 2 ** 30
    return float(round_bits(round_bits(fn(arg), 64), 53))


def hexlist(vals, per_line=3):
    items = [float.hex(v) for v in vals]
    lines = []
    for i in range(0, len(items), per_line):
        lines.append("  " + ", ".join(items[i:i + per_line]) + ",")
    return "\n".join(lines)


def main(out=sys.stdout):
    tan = [x87(mp.tan, i * 0x100000 - 0xff00000) for i in range(511)]
    sin = [x87(mp.sin, i * 0x100000 - 0xff80000) for i in range(512)]
    cos = [x87(mp.cos, i * 0x100000 - 0xff80000) for i in range(512)]
    quad = []
    for a in (0, 0x20000000, 0x40000000, 0x60000000):
        quad += [x87(mp.cos, a), x87(mp.sin, a)]
    c64 = round_bits(mp.mpf(2 ** 30) / PI64, 64)
    c_hi = float(c64)
    c_lo = float(c64 - mp.mpf(c_hi))
    w = out.write
    w("/* Generated by gen_angle_tables.py -- do not edit. */\n")
    w("#ifndef WB_ANGLE_TABLES_H\n#define WB_ANGLE_TABLES_H\n")
    w("static const double kWbTan[511] = {\n" + hexlist(tan) + "\n};\n")
    w("static const double kWbSin[512] = {\n" + hexlist(sin) + "\n};\n")
    w("static const double kWbCos[512] = {\n" + hexlist(cos) + "\n};\n")
    w("/* cos, sin of 0, 90, 180, 270 degrees as the reference's long double gives them */\n")
    w("static const double kWbQuadrantCosSin[8] = {\n" + hexlist(quad, 2) + "\n};\n")
    w("/* 0x40000000 / M_PIl in 64-bit long double, as hi + lo doubles */\n")
    w(f"#define WB_ATAN_SCALE_HI {float.hex(c_hi)}\n#define WB_ATAN_SCALE_LO {float.hex(c_lo)}\n")
    w("#endif\n")


if __name__ == "__main__":
    main()
