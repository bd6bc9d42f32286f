"""Generates cafe_crmath_tables.h: double-double tables for cafe_crmath.h.

Run from this folder with mpmath available (it ships with sympy):
    python gen_crmath_tables.py > cafe_crmath_tables.h
Each entry v is split as hi = RN(v), lo = RN(v - hi), from 300-bit values.
"""
import mpmath

mpmath.mp.prec = 300


def split(v):
    hi = float(mpmath.mpf(v))
    hi = mpmath.libmp.to_float(mpmath.mpf(v)._mpf_, rnd="n")
    lo = mpmath.libmp.to_float((mpmath.mpf(v) - mpmath.mpf(hi))._mpf_, rnd="n")
    return hi, lo


def hx(x):
    return float.hex(x)


def main():
    out = []
    out.append("// Generated by gen_crmath_tables.py -- do not edit.")
    out.append("// Double-double tables: value = hi + lo, |lo| <= ulp(hi)/2.")
    out.append("#ifndef CAFE_CRMATH_TABLES_H")
    out.append("#define CAFE_CRMATH_TABLES_H")
    out.append("#define CRM_ATAN_STEPS 64")
    out.append("#define CRM_SC_STEPS 128")
    rows = []
    for k in range(65):
        h, l = split(mpmath.atan(mpmath.mpf(k) / 64))
        rows.append("  {%s, %s}," % (hx(h), hx(l)))
    out.append("CRM_TABLE_DECL(double, crm_atan_tab, [65][2]) = {")
    out += rows
    out.append("};")
    rows = []
    for j in range(104):
        x = mpmath.mpf(j) / 128
        sh, sl = split(mpmath.sin(x))
        ch, cl = split(mpmath.cos(x))
        rows.append("  {%s, %s, %s, %s}," % (hx(sh), hx(sl), hx(ch), hx(cl)))
    out.append("CRM_TABLE_DECL(double, crm_sincos_tab, [104][4]) = {")
    out += rows
    out.append("};")
    pio2 = mpmath.pi / 2
    p1 = mpmath.libmp.to_float(pio2._mpf_, rnd="n")
    p2 = mpmath.libmp.to_float((pio2 - p1)._mpf_, rnd="n")
    p3 = mpmath.libmp.to_float((pio2 - p1 - p2)._mpf_, rnd="n")
    p4 = mpmath.libmp.to_float((pio2 - p1 - p2 - p3)._mpf_, rnd="n")
    pih, pil = split(mpmath.pi)
    out.append("#define CRM_PIO2_1 %s" % hx(p1))
    out.append("#define CRM_PIO2_2 %s" % hx(p2))
    out.append("#define CRM_PIO2_3 %s" % hx(p3))
    out.append("#define CRM_PIO2_4 %s" % hx(p4))
    out.append("#define CRM_PI_HI %s" % hx(pih))
    out.append("#define CRM_PI_LO %s" % hx(pil))
    out.append("#define CRM_TWO_OVER_PI %s" % hx(mpmath.libmp.to_float((2 / mpmath.pi)._mpf_, rnd="n")))
    # exp: x = k ln2/128 + r, exp(x) = 2^(k>>7) 2^((k&127)/128) exp(r)
    c = mpmath.log(2) / 128

    def round_bits(v, bits):
        return mpmath.libmp.to_float(mpmath.libmp.normalize(*mpmath.mpf(v)._mpf_[:3], mpmath.mpf(v)._mpf_[3],
                                                            bits, "n"), rnd="n")

    l1 = round_bits(c, 35)
    l2 = round_bits(c - l1, 35)
    l3 = mpmath.libmp.to_float((c - l1 - l2)._mpf_, rnd="n")
    out.append("#define CRM_EXP_STEPS 128")
    out.append("#define CRM_LN2_128_1 %s" % hx(l1))
    out.append("#define CRM_LN2_128_2 %s" % hx(l2))
    out.append("#define CRM_LN2_128_3 %s" % hx(l3))
    out.append("#define CRM_INV_LN2_128 %s" % hx(mpmath.libmp.to_float((128 / mpmath.log(2))._mpf_, rnd="n")))
    rows = []
    for j in range(128):
        h, l = split(mpmath.power(2, mpmath.mpf(j) / 128))
        rows.append("  {%s, %s}," % (hx(h), hx(l)))
    out.append("CRM_TABLE_DECL(double, crm_exp2_tab, [128][2]) = {")
    out += rows
    out.append("};")
    for n, name in ((3, "6"), (4, "24")):
        h, l = split(1 / mpmath.factorial(n))
        out.append("#define CRM_INV_FACT%s_HI %s" % (name, hx(h)))
        out.append("#define CRM_INV_FACT%s_LO %s" % (name, hx(l)))
    out.append("#endif")
    print("\n".join(out))


if __name__ == "__main__":
    main()
