"""Generate pf7_series.cuh: the Taylor series, in eps = x - 1, of the exact
real-arithmetic output of powfancy7th (src/gpukernels_sph.jl:499-515 -- the
bit-trick first guess followed by two Halley steps t <- t - t(t^7-x)/(4t^7+3x)).

The density-diffusion term only ever calls powfancy7th on x = 1 + eps with a
small eps (rho0*g*dz/Cb), where the bit-trick guess is an affine function of x
on each side of 1 (one binade each) and the two Halley steps are a fixed
rational function of x.  Its Taylor series, computed here in exact rational
arithmetic, reproduces that rational function -- including the iteration's own
small bias against the true 7th root -- to far below one ulp for |eps| <=
EPS_MAX, at the cost of one polynomial instead of two divisions per call.

Run:  python gen_pf7_series.py   (writes pf7_series.cuh beside this file)
"""
from fractions import Fraction as F
import os
import struct

K = 10            # highest power kept in the exact series
EPS_MAX = F(1, 128)
EPS_SHORT = F(1, 1024)  # a shorter head of the same series serves |eps| <= EPS_SHORT
TOL = 2.0 ** -64  # dropped tail, relative to 1


def smul(a, b):
    out = [F(0)] * (K + 1)
    for i, ai in enumerate(a):
        if ai == 0:
            continue
        for j in range(K + 1 - i):
            out[i + j] += ai * b[j]
    return out


def sinv(a):
    # 1/a as a truncated series (a[0] != 0)
    out = [F(0)] * (K + 1)
    out[0] = 1 / a[0]
    for n in range(1, K + 1):
        s = sum(a[i] * out[n - i] for i in range(1, n + 1))
        out[n] = -s / a[0]
    return out


def halley(t, x):
    t2 = smul(t, t)
    t4 = smul(t2, t2)
    t7 = smul(smul(t4, t2), t)
    num = smul(t, [a - b for a, b in zip(t7, x)])
    den = [4 * a + 3 * b for a, b in zip(t7, x)]
    corr = smul(num, sinv(den))
    return [a - b for a, b in zip(t, corr)]


def first_guess(upper):
    # real-valued model of 0x36cd000000000000 + bits(x) / 7 reinterpreted as a
    # double, x = 1 + eps;  upper: x in [1, 2), bits = 0x3FF0.. + eps 2^52;
    # lower: x in [0.5, 1), bits = 0x3FE0.. + (1 + 2 eps) 2^52.  The guess
    # keeps one exponent over |eps| <= EPS_MAX (checked), so it is affine there.
    two52 = F(2) ** 52
    C = F(0x36CD000000000000)
    if upper:
        base, slope = F(0x3FF0000000000000), two52
    else:
        base, slope = F(0x3FE0000000000000) + two52, 2 * two52
    ends = [C + (base + slope * e) / 7 for e in ((0, EPS_MAX) if upper else (-EPS_MAX, 0))]
    ex = {int(v) >> 52 for v in ends}
    assert len(ex) == 1, "first guess changes exponent inside the range"
    ex = ex.pop()
    scale = F(2) ** (ex - 1023) if ex >= 1023 else F(1, 2 ** (1023 - ex))
    t0 = C + base / 7  # bits of the guess at eps = 0
    a = scale * (1 + (t0 - ex * two52) / two52)
    b = scale * (slope / 7) / two52
    return [a, b] + [F(0)] * (K - 1)


def series(upper):
    x = [F(1), F(1)] + [F(0)] * (K - 1)
    t = first_guess(upper)
    t = halley(t, x)
    t = halley(t, x)
    s = list(t)
    s[0] -= 1  # s = t - 1
    n = K
    while n > 1 and abs(float(s[n])) * float(EPS_MAX) ** n < TOL:
        n -= 1
    assert abs(float(s[K])) * float(EPS_MAX) ** K < TOL, "raise K"
    return [float(c) for c in s[: n + 1]]


def ref_pf7(x):
    ax = abs(x)
    b = struct.unpack("<Q", struct.pack("<d", ax))[0]
    b = 0x36CD000000000000 + b // 7
    t = struct.unpack("<d", struct.pack("<Q", b))[0]
    t = t if x >= 0 else -t
    for _ in range(2):
        t2 = t * t
        t3 = t2 * t
        t4 = t2 * t2
        xot4 = x / t4
        t = t - (t * (t3 - xot4)) / (4.0 * t3 + 3.0 * xot4)
    return t


def horner(c, e):
    r = 0.0
    for a in reversed(c):
        r = r * e + a
    return r


def short_terms(c):
    """Terms of series c that matter for |eps| <= EPS_SHORT (the dropped
    tail stays below TOL relative to 1)."""
    n = len(c) - 1
    while n > 1 and abs(c[n]) * float(EPS_SHORT) ** n < TOL:
        n -= 1
    return n + 1


def sweep(up, lo, eps_max, n):
    """Largest gap to the iteration's own output over a sweep of |eps| <=
    eps_max, with the first n terms of each series."""
    worst = 0.0
    for i in range(-2000, 2001):
        e = float(eps_max) * i / 2000.0
        x = 1.0 + e
        e = x - 1.0
        s = horner((up if e >= 0 else lo)[:n], e)
        worst = max(worst, abs((1.0 + s) - ref_pf7(x)))
    return worst


def main():
    up, lo = series(True), series(False)
    worst = sweep(up, lo, EPS_MAX, max(len(up), len(lo)))
    assert worst <= 4.5e-16, worst
    nshort = max(short_terms(up), short_terms(lo))
    worst_short = sweep(up, lo, EPS_SHORT, nshort)
    assert worst_short <= 4.5e-16, worst_short
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "pf7_series.cuh"), "w") as f:
        f.write("// Generated by gen_pf7_series.py -- do not edit.\n")
        f.write("// powfancy7th(1 + eps) - 1 as a polynomial in eps, |eps| <= PF7_EPS_MAX\n")
        f.write("// (src/gpukernels_sph.jl:499-515; worst gap to the iteration over a sweep: %.3g)\n" % worst)
        f.write("#pragma once\n")
        f.write("#define PF7_EPS_MAX %r\n" % float(EPS_MAX))
        f.write("// |eps| <= PF7_EPS_SHORT needs only the first PF7_SHORT_N terms (worst gap %.3g)\n" % worst_short)
        f.write("#define PF7_EPS_SHORT %r\n" % float(EPS_SHORT))
        f.write("#define PF7_SHORT_N %d\n" % nshort)
        for name, c in (("PF7_UP", up), ("PF7_LO", lo)):
            f.write("#define %s_N %d\n" % (name, len(c)))
            f.write("#define %s_C {%s}\n" % (name, ", ".join(repr(v) for v in c)))
    print("pf7 series:", len(up), len(lo), "terms; worst gap", worst, "; short head", nshort, "terms, gap",
          worst_short)


if __name__ == "__main__":
    main()
