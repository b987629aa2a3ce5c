"""Writes nf_math_tables.h: the tables of the table-driven logarithm and exponential in
nf_math.h (Tang's method: P. T. P. Tang, "Table-driven implementation of the exponential
function in IEEE floating-point arithmetic", ACM TOMS 15 (1989) 144-157, and "... of the
logarithm function", ACM TOMS 16 (1990) 378-400).

Every value is computed here at 200 bits with mpmath and rounded to the nearest double (the
low halves are the rounded remainders), so the tables are exact restatements of their
definitions:

  log table, 128 entries for z in [LOG_OFF, 2 LOG_OFF) split by the 7 bits below z's exponent
  field after subtracting LOG_OFF's bit pattern: invc = the double nearest 1/c for c the
  middle of entry j's bit range (invc = 1 exactly for the entry centred on 1.0), and
  -log(invc) as hi + lo, so that log z = -log(invc) + log1p(z invc - 1) holds exactly for the
  stored invc.
  exp table, 128 entries: 2^(j/128) as hi + lo.

Run it from this directory: python gen_nf_math_tables.py > nf_math_tables.h
"""
import struct

import mpmath

mpmath.mp.prec = 200

LOG_OFF = 0x3FE6900000000000      # 1.0's bit pattern minus 75.5 entries of 2^45
ENTRIES = 128


def from_bits(u: int) -> float:
    return struct.unpack("<d", struct.pack("<Q", u))[0]


def nearest(v) -> float:
    """The double nearest v (mpmath value), checked to be within half an ulp."""
    f = float(v)
    if f != 0.0:
        import math
        assert abs(mpmath.mpf(f) - v) <= mpmath.mpf(math.ulp(f)) / 2
    return f


def split(v):
    hi = nearest(v)
    lo = nearest(v - mpmath.mpf(hi))
    return hi, lo


def log_entries():
    rows = []
    for j in range(ENTRIES):
        centre = from_bits(LOG_OFF + j * (1 << 45) + (1 << 44))
        if centre == 1.0:
            rows.append((1.0, 0.0, 0.0))
            continue
        invc = nearest(1 / mpmath.mpf(centre))
        hi, lo = split(-mpmath.log(mpmath.mpf(invc)))
        rows.append((invc, hi, lo))
    return rows


def exp_entries():
    return [split(mpmath.power(2, mpmath.mpf(j) / ENTRIES)) for j in range(ENTRIES)]


def main():
    ln2 = mpmath.log(2)
    step = ln2 / ENTRIES
    l_hi = mpmath.nint(step * mpmath.mpf(2) ** 42) / mpmath.mpf(2) ** 42   # 35 bits
    l_hi = nearest(l_hi)
    l_lo = nearest(step - mpmath.mpf(l_hi))
    inv = nearest(ENTRIES / ln2)
    out = ["/* Generated by gen_nf_math_tables.py; do not edit. */",
           "#ifndef NF_MATH_TABLES_H", "#define NF_MATH_TABLES_H", "",
           f"#define NF_LOG_OFF 0x{LOG_OFF:016x}ULL",
           f"#define NF_EXP_N_OVER_LN2 {inv.hex()}   /* 128 / ln 2 */",
           f"#define NF_EXP_L_HI {l_hi.hex()}   /* ln 2 / 128, 35 significant bits */",
           f"#define NF_EXP_L_LO {l_lo.hex()}", "",
           "/* invc, -log(invc) hi, lo, 0 */", "#define NF_LOG_TABLE \\"]
    for invc, hi, lo in log_entries():
        out.append(f"    {invc.hex()}, {hi.hex()}, {lo.hex()}, 0.0, \\")
    out += ["", "/* 2^(j/128) hi, lo */", "#define NF_EXP_TABLE \\"]
    for hi, lo in exp_entries():
        out.append(f"    {hi.hex()}, {lo.hex()}, \\")
    out += ["", "#endif /* NF_MATH_TABLES_H */"]
    print("\n".join(out))


if __name__ == "__main__":
    main()
