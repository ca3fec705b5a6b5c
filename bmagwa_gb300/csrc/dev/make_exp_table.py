"""Writes exp_table.h: 2^(i/256), i = 0..255, each rounded to the nearest
double (60-digit decimal arithmetic, then Python's correctly rounded
string-to-float conversion), and the same values as FP32 pairs (hi = the
nearest float, lo = the nearest float to the remainder).  Run from this
directory."""
import struct
from decimal import Decimal, getcontext

getcontext().prec = 60
ln2 = Decimal(2).ln()
exact = [(ln2 * i / 256).exp() for i in range(256)]
vals = [float(str(x)) for x in exact]


def f32(x):
    return struct.unpack("f", struct.pack("f", float(str(x))))[0]


pairs = []
for x in exact:
    hi = f32(x)
    pairs += [hi, f32(x - Decimal(hi))]
lines = ["// 2^(i/256), i = 0..255, rounded to the nearest double (make_exp_table.py)",
         "#ifndef BMG_EXP_TABLE_H_", "#define BMG_EXP_TABLE_H_", "",
         "static __device__ const double kExp2Tab[256] = {"]
for i in range(0, 256, 4):
    lines.append("  " + ", ".join(v.hex() for v in vals[i:i + 4]) + ",")
lines += ["};", "", "// 2^(i/256) as FP32 pairs: entries 2i (hi) and 2i + 1 (lo)",
          "static __device__ const float kExp2TabF[512] = {"]
for i in range(0, 512, 4):
    lines.append("  " + ", ".join(v.hex() + "f" for v in pairs[i:i + 4]) + ",")
lines += ["};", "", "#endif", ""]
open("exp_table.h", "w").write("\n".join(lines))
