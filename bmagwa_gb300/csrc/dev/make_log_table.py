"""Writes log_table.h, the tables of flog.h's table-driven logarithm: for
j = 0..255, r_j = the double nearest to 1 / (1 + j/256), and
T_j = -log(r_j) as the sum of two doubles (hi = nearest double, lo =
nearest double to the remainder), from 60-digit decimal arithmetic and
Python's correctly rounded string-to-float conversion.  Run from this
directory."""
import struct
from decimal import Decimal, getcontext

getcontext().prec = 60
rs, ts = [], []
for j in range(256):
    r = float(str(Decimal(1) / (Decimal(1) + Decimal(j) / 256)))
    t = -Decimal(r).ln()  # Decimal(r) is the double's exact value
    hi = float(str(t))
    lo = float(str(t - Decimal(hi)))
    rs.append(r)
    ts += [hi, lo]
lines = ["// Tables of flog.h (make_log_table.py): r_j = 1 / (1 + j/256) rounded to the",
         "// nearest double; -log(r_j) as hi + lo doubles (entries 2j, 2j + 1)",
         "#ifndef BMG_LOG_TABLE_H_", "#define BMG_LOG_TABLE_H_", "",
         "static __device__ const double kLogR[256] = {"]
for i in range(0, 256, 4):
    lines.append("  " + ", ".join(v.hex() for v in rs[i:i + 4]) + ",")
lines += ["};", "", "static __device__ const double kLogT[512] = {"]
for i in range(0, 512, 4):
    lines.append("  " + ", ".join(v.hex() for v in ts[i:i + 4]) + ",")
# ln 2 as hi + lo, hi with its 11 lowest bits clear so that e * hi is exact
# for every binary exponent e of a double
hi2 = float(str(Decimal(2).ln()))
b = struct.unpack("<Q", struct.pack("<d", hi2))[0] & ~((1 << 11) - 1)
hi2 = struct.unpack("<d", struct.pack("<Q", b))[0]
lo2 = float(str(Decimal(2).ln() - Decimal(hi2)))
lines += ["};", "", "#define BMG_LN2_HI " + hi2.hex(), "#define BMG_LN2_LO " + lo2.hex(), "", "#endif", ""]
open("log_table.h", "w").write("\n".join(lines))
