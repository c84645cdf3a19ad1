"""Generate gfm_tables.h: the constant tables of the table-driven exp/log
and of the fixed-point pow.

The elementary functions follow P. T. P. Tang, "Table-driven implementation of
the exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2),
1989, and "Table-driven implementation of the logarithm function in IEEE
floating-point arithmetic", ACM TOMS 16(4), 1990: a table lookup reduces the
argument to a short interval on which a low-degree polynomial suffices.  The
tables are computed here at 60 significant digits with mpmath and rounded to
the nearest double, so the header is reproducible:

    python gen_tables.py > gfm_tables.h
"""
import mpmath

mpmath.mp.dps = 60


def d(x):
    """Round an mpmath value to the nearest double and print it exactly."""
    return float(x).hex()


def main():
    out = []
    out.append("// Generated by gen_tables.py (mpmath, 60 digits). Do not edit.")
    out.append("#pragma once")
    out.append("// 2^(j/64), j = 0..63")
    out.append("#define GFM_EXP2_TABLE { \\")
    for j in range(64):
        out.append(f"  {d(mpmath.power(2, mpmath.mpf(j) / 64))}, \\")
    out.append("}")
    out.append("// log(1 + j/128), j = -32..64 (index j + 32)")
    out.append("#define GFM_LOGF_TABLE { \\")
    for j in range(-32, 65):
        out.append(f"  {d(mpmath.log(1 + mpmath.mpf(j) / 128))}, \\")
    out.append("}")
    out.append("// 1 / (1 + j/128), j = -32..64 (index j + 32)")
    out.append("#define GFM_INVF_TABLE { \\")
    for j in range(-32, 65):
        out.append(f"  {d(1 / (1 + mpmath.mpf(j) / 128))}, \\")
    out.append("}")
    ln2 = mpmath.log(2)
    # ln2/64 split: hi keeps 32 significant bits so k*hi is exact for |k| < 2^20.
    step = ln2 / 64
    hi = mpmath.mpf(int(mpmath.floor(step * 2 ** 38))) / 2 ** 38
    lo = step - hi
    out.append(f"#define GFM_LN2_64_HI {d(hi)}")
    out.append(f"#define GFM_LN2_64_LO {d(lo)}")
    out.append(f"#define GFM_INV_LN2_64 {d(64 / ln2)}")
    hi2 = mpmath.mpf(int(mpmath.floor(ln2 * 2 ** 40))) / 2 ** 40
    out.append(f"#define GFM_LN2_HI {d(hi2)}")
    out.append(f"#define GFM_LN2_LO {d(ln2 - hi2)}")
    out.append(f"#define GFM_PI {d(mpmath.pi)}")
    out.append(f"#define GFM_PI_2 {d(mpmath.pi / 2)}")
    # Fixed-point pow (gfm_pow): log2 by two table reductions m R1 R2 = 1 + r
    # (R1 = RI1/2^16 ~ 1/(1 + j/64), j = -16..32; R2 = RI2/2^24 ~
    # 1/(1 + k/4096), k = -48..48) with log2(1/R1), log2(1/R2) in Q62 and
    # 1/ln2 in Q62; exp2 by 2^(j/64) in Q63 (j = 0..63), 2^(k/4096) - 1 in
    # Q64 (k = 0..63) and ln2 in Q64.
    def nint(v):
        return int(mpmath.nint(v))
    two = mpmath.mpf(2)
    ri1 = [nint(two ** 16 / (1 + mpmath.mpf(j) / 64)) for j in range(-16, 33)]
    ri2 = [nint(two ** 24 / (1 + mpmath.mpf(k) / 4096)) for k in range(-48, 49)]
    out.append("// RI1_j = round(2^16 / (1 + j/64)), j = -16..32 (index j + 16)")
    out.append("#define GFM_XLOG1_RI { \\")
    out += [f"  {v}u, \\" for v in ri1]
    out.append("}")
    out.append("// round(log2(2^16 / RI1_j) * 2^62)")
    out.append("#define GFM_XLOG1_T { \\")
    out += [f"  {nint(mpmath.log(two ** 16 / v, 2) * two ** 62)}LL, \\" for v in ri1]
    out.append("}")
    out.append("// RI2_k = round(2^24 / (1 + k/4096)), k = -48..48 (index k + 48)")
    out.append("#define GFM_XLOG2_RI { \\")
    out += [f"  {v}u, \\" for v in ri2]
    out.append("}")
    out.append("// round(log2(2^24 / RI2_k) * 2^62)")
    out.append("#define GFM_XLOG2_T { \\")
    out += [f"  {nint(mpmath.log(two ** 24 / v, 2) * two ** 62)}LL, \\" for v in ri2]
    out.append("}")
    out.append(f"#define GFM_XLOG_INVLN2 {nint(two ** 62 / ln2)}LL   // round(2^62 / ln 2)")
    out.append("// round(2^(j/64) * 2^63), j = 0..63")
    out.append("#define GFM_XEXP1_E { \\")
    out += [f"  {nint(mpmath.power(2, mpmath.mpf(j) / 64) * two ** 63)}ULL, \\" for j in range(64)]
    out.append("}")
    out.append("// round((2^(k/4096) - 1) * 2^64), k = 0..63")
    out.append("#define GFM_XEXP2_E { \\")
    out += [f"  {nint((mpmath.power(2, mpmath.mpf(k) / 4096) - 1) * two ** 64)}ULL, \\" for k in range(64)]
    out.append("}")
    out.append(f"#define GFM_XEXP_LN2 {nint(ln2 * two ** 64)}ULL   // round(2^64 ln 2)")
    # Taylor coefficients of asin(x) = sum c_n x^(2n+1), n = 0..27
    out.append("#define GFM_ASIN_COEFFS { \\")
    for n in range(28):
        c = mpmath.factorial(2 * n) / (4 ** n * mpmath.factorial(n) ** 2 * (2 * n + 1))
        out.append(f"  {d(c)}, \\")
    out.append("}")
    print("\n".join(out))


if __name__ == "__main__":
    main()
