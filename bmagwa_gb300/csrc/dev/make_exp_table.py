"""Writes exp_table.h: 2^(i/256), i = 0..255, each rounded to the nearest
double (60-digit decimal arithmetic, then Python's correctly rounded
string-to-float conversion).  Run from this directory."""
from decimal import Decimal, getcontext

getcontext().prec = 60
ln2 = Decimal(2).ln()
vals = [float(str((ln2 * i / 256).exp())) for i in range(256)]
lines = ["// 2^(i/256), i = 0..255, rounded to the nearest double (make_exp_table.py)",
         "#ifndef BMG_EXP_TABLE_H_", "#define BMG_EXP_TABLE_H_", "",
         "static __device__ const double kExp2Tab[256] = {"]
for i in range(0, 256, 4):
    lines.append("  " + ", ".join(v.hex() for v in vals[i:i + 4]) + ",")
lines += ["};", "", "#endif", ""]
open("exp_table.h", "w").write("\n".join(lines))
