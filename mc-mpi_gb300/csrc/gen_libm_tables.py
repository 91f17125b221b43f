#!/usr/bin/env python3
"""Generate libm_tables.inc: the constant tables of the float-float logf/expf
evaluators in exact_libm.h.

Every value here is derived from the mathematics with mpmath at 60 digits and
rounded to binary32 (or split into a binary32 float-float pair).  The layout:

  log:  x = 2^k * m, m in [0.75, 1.5).  The mantissa's top 7 bits pick bucket i
        (128 buckets over [1, 2); buckets 64..127 are halved into [0.75, 1)).
        invc_i = 1/c_i rounded to 8 significant bits, c_i the bucket centre,
        except buckets 0 and 127 (next to 1.0) which use c = invc = 1 so that
        log(x) near 1 is the pure log1p polynomial.  8 significant bits make
        r = m*invc - 1 exact in one fma.  L_i = -log(invc_i) as hi + lo.
        ln2 = LN2_HI + LN2_MID + LN2_LO with 16 + 16 + 24 significant bits, so
        k*LN2_HI and k*LN2_MID are exact for |k| < 256.
  exp:  t = (64*q + j) * ln2/64 + r, |r| <= ln2/128.  T_j = 2^(j/64) as hi + lo.
        ln2/64 = C1 + C2 + C3 with 10 + 24 + 24 significant bits (k*C1 exact for
        |k| < 2^14).

Run:  python3 gen_libm_tables.py > libm_tables.inc

The output defines the scalar constants as macros and MCG_LIBM_TAB_INIT, the
initializer of struct mcg_libm_tab (exact_libm.h).
"""
import struct
import mpmath

mpmath.mp.prec = 200


def f32(v):
    """Round an mpmath number to the nearest binary32 (ties to even)."""
    v = mpmath.mpf(v)
    if v == 0:
        return 0.0
    # binary32: 24 significant bits; all values here are normal.
    e = int(mpmath.floor(mpmath.log(abs(v), 2)))
    scale = mpmath.mpf(2) ** (23 - e)
    n = v * scale
    fl = mpmath.floor(n)
    rem = n - fl
    if rem > 0.5 or (rem == 0.5 and int(fl) % 2 == 1):
        fl += 1
    out = float(fl / scale)
    assert struct.unpack("<f", struct.pack("<f", out))[0] == out
    return out


def round_bits(v, bits):
    """Round to `bits` significant bits (ties to even)."""
    v = mpmath.mpf(v)
    e = int(mpmath.floor(mpmath.log(abs(v), 2)))
    scale = mpmath.mpf(2) ** (bits - 1 - e)
    n = v * scale
    fl = mpmath.floor(n)
    rem = n - fl
    if rem > 0.5 or (rem == 0.5 and int(fl) % 2 == 1):
        fl += 1
    return mpmath.mpf(fl) / scale


def split(v):
    hi = f32(v)
    lo = f32(mpmath.mpf(v) - mpmath.mpf(hi))
    return hi, lo


def hexf(x):
    return float(x).hex()


def fl(x):
    return f"{hexf(x)}f"


out = []
out.append("/* Generated by gen_libm_tables.py; do not edit. Values derived with mpmath. */")
# ---- log ----
out.append("#define MCG_LOG_NB 128")
invcs, lhis, llos = [], [], []
for i in range(128):
    if i == 0 or i == 127:
        invc = mpmath.mpf(1)
    else:
        c = 1 + (mpmath.mpf(i) + mpmath.mpf("0.5")) / 128
        if i >= 64:
            c = c / 2
        invc = round_bits(1 / c, 8)
    L = -mpmath.log(invc)
    hi, lo = split(L) if L != 0 else (0.0, 0.0)
    invcs.append(float(invc))
    lhis.append(hi)
    llos.append(lo)
ln2 = mpmath.log(2)
h16 = round_bits(ln2, 16)
m16 = round_bits(ln2 - h16, 16)
l24 = f32(ln2 - h16 - m16)
out.append(f"#define MCG_LN2_HI {fl(float(h16))}")
out.append(f"#define MCG_LN2_MID {fl(float(m16))}")
out.append(f"#define MCG_LN2_LO {fl(l24)}")
# log1p polynomial coefficients (Taylor, from the series)
for n, name in [(3, "P3"), (4, "P4"), (5, "P5"), (6, "P6")]:
    sign = 1 if n % 2 == 1 else -1
    out.append(f"#define MCG_LOG_{name} {fl(f32(mpmath.mpf(sign) / n))}")

# ---- exp ----
out.append("#define MCG_EXP_NT 64")
this, tlos = [], []
for j in range(64):
    v = mpmath.mpf(2) ** (mpmath.mpf(j) / 64)
    hi, lo = split(v)
    this.append(hi)
    tlos.append(lo)
c = ln2 / 64
c1 = round_bits(c, 10)
c2 = f32(c - c1)
c3 = f32(c - c1 - mpmath.mpf(c2))
out.append(f"#define MCG_EXP_C1 {fl(float(c1))}")
out.append(f"#define MCG_EXP_C2 {fl(c2)}")
out.append(f"#define MCG_EXP_C3 {fl(c3)}")
out.append(f"#define MCG_EXP_INV {fl(f32(64 / ln2))}")
for n, name in [(3, "Q3"), (4, "Q4")]:
    out.append(f"#define MCG_EXP_{name} {fl(f32(1 / mpmath.factorial(n)))}")
# one initializer for the mcg_libm_tab struct of exact_libm.h
out.append("#define MCG_LIBM_TAB_INIT { \\")
for name, vals in [("log_invc", invcs), ("log_lhi", lhis), ("log_llo", llos),
                   ("exp_thi", this), ("exp_tlo", tlos)]:
    out.append("  { " + ", ".join(fl(v) for v in vals) + " }, \\")
out.append("}")
print("\n".join(out))
