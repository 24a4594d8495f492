"""Generates sh_basis.inc: the real spherical-harmonics basis up to degree 8 as FP32
polynomials in the Cartesian components (x, y, z) of a unit direction.

Convention (the one tiny-cuda-nn's SphericalHarmonicsEncoding uses,
rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/encodings/spherical_harmonics.h:46-151):
output index l*l + l + m for m in [-l, l];
    m > 0:  sqrt(2) K_l^m cos(m phi) P_l^m(cos theta)
    m < 0:  sqrt(2) K_l^|m| sin(|m| phi) P_l^|m|(cos theta)
    m = 0:  K_l^0 P_l^0(cos theta)
with K_l^m = sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!) and P_l^m carrying the Condon-Shortley
phase (-1)^m.  On the unit sphere r^l Y is a homogeneous polynomial; this script derives it
symbolically (sympy) and prints one C expression per basis function.

Run:  python neural_lod_gb300/csrc/gen_sh.py > neural_lod_gb300/csrc/sh_basis.inc
"""
import sympy as sp

x, y, z = sp.symbols("x y z", real=True)


def assoc_legendre_poly(l, m):
    """P_l^m(cos theta) / sin^m(theta), times the Condon-Shortley phase (-1)^m, as a polynomial
    in z = cos theta (Rodrigues' formula).  It is deliberately not homogenised with
    r^2 = x^2 + y^2 + z^2: the z-polynomial times Re/Im (x + i y)^m is the form tiny-cuda-nn
    evaluates, so inputs slightly off the unit sphere give the same values."""
    t = sp.symbols("t")
    p = sp.diff((t * t - 1) ** l, t, l + m) / (2 ** l * sp.factorial(l))
    p = sp.expand((-1) ** m * p)
    return sp.expand(p.subs(t, z))


def basis(l, m):
    am = abs(m)
    K = sp.sqrt(sp.Rational(2 * l + 1, 4) / sp.pi * sp.factorial(l - am) / sp.factorial(l + am))
    leg = assoc_legendre_poly(l, am)
    # sin^m(theta) cos(m phi) = Re((x + i y)^m), sin^m sin(m phi) = Im((x + i y)^m)
    c = sp.expand((x + sp.I * y) ** am)
    if m > 0:
        ang = sp.sqrt(2) * sp.re(c)
    elif m < 0:
        ang = sp.sqrt(2) * sp.im(c)
    else:
        ang = sp.Integer(1)
    return sp.expand(K * leg * ang)


def to_c(expr):
    """FP32 C expression: a sum of monomials with FP32 literal coefficients."""
    expr = sp.expand(expr)
    terms = []
    for monom, coef in sp.Poly(expr, x, y, z).terms():
        c = sp.N(coef, 20)
        parts = []
        for v, e in zip(("x", "y", "z"), monom):
            parts += [v] * e
        terms.append((float(c), parts))
    out = []
    for c, parts in terms:
        s = "%.17gf" % c
        if parts:
            s += "*" + "*".join(parts)
        out.append(s)
    return " + ".join(out).replace("+ -", "- ")


def main():
    print("// Generated by gen_sh.py: real spherical harmonics up to degree 8 (unit directions).")
    print("// Defines SH_BASIS(OUT, x, y, z, degree): OUT(i, value) for i in [0, degree^2).")
    print("#define SH_BASIS(OUT, x, y, z, degree) do { \\")
    for l in range(8):
        if l > 0:
            print("  if ((degree) <= %d) break; \\" % l)
        for m in range(-l, l + 1):
            idx = l * l + l + m
            print("  OUT(%d, (%s)); \\" % (idx, to_c(basis(l, m))))
    print("} while (0)")


if __name__ == "__main__":
    main()
