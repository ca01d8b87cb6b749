"""Coefficients of the GELU used by the tcgen05 inference epilogue (pt_mlp.cu).

GELU(z) = z * Phi(z), Phi the standard normal CDF.  With a = min(|z|, A),
A = 4 * sqrt(2), and e = Phi(-a) = erfc(a / sqrt(2)) / 2:

    GELU(z) = max(z, 0) - a * e

exactly for |z| <= A (for z >= 0, z - z Phi(-z) = z Phi(z); for z < 0, -|z| Phi(z) =
z Phi(z)), and within 4.4e-8 of it beyond (Phi(-A) = 7.7e-9).  e is evaluated as
2^p(-a), p a degree-7 polynomial fitted here to log2(erfc(a / sqrt(2)) / 2) on
[0, A] in the variable n = -a: one exp2 (ex2.approx) and seven fused multiply-adds,
which the kernel runs two lanes at a time (fma.rn.f32x2).  The form has no
cancellation for negative z, unlike 0.5 z (1 + erf(z / sqrt 2)).

The fit is a weighted least-squares fit on a Chebyshev basis, reweighted toward the
minimax error of e (iteratively reweighted least squares), then converted to
monomials in n.  The script checks the float32 Horner evaluation (with single
rounding per fused multiply-add) against the exact e and prints the C table.

    python pandemicthrust_gb300/csrc/fit_gelu.py
"""
import numpy as np
from numpy.polynomial import chebyshev as C
from numpy.polynomial import polynomial as P
from scipy.special import erfc

DEGREE = 7
A = 4.0 * np.sqrt(2.0)


def f32(x):
    return np.asarray(x, np.float64).astype(np.float32).astype(np.float64)


def fit():
    a = np.linspace(0.0, A, 400001)
    e = 0.5 * erfc(a / np.sqrt(2.0))
    target = np.log2(e)
    t = 2.0 * a / A - 1.0            # Chebyshev variable on [0, A]
    w = e.copy()                      # absolute error of e = e ln2 * error of log2 e
    for _ in range(40):
        c = C.chebfit(t, target, DEGREE, w=w)
        err = np.abs(C.chebval(t, c) - target) * e
        w = w * (1.0 + err / err.max())
    # monomials in t, then in n = -a: t = 2a/A - 1 = -(2/A) n - 1
    mono_t = C.cheb2poly(c)
    mono_n = P.Polynomial(mono_t)(P.Polynomial([-1.0, -2.0 / A])).coef
    return f32(mono_n)


def horner32(coef, n):
    acc = np.full_like(n, coef[-1])
    for k in range(len(coef) - 2, -1, -1):
        acc = f32(acc * n + coef[k])  # one rounding per fused multiply-add
    return acc


def check(coef):
    z = np.linspace(-12.0, 12.0, 2_000_001)
    a = f32(np.minimum(np.abs(z), f32(A)))
    e = 2.0 ** horner32(coef, -a)
    gelu = np.maximum(z, 0.0) - a * e
    exact = 0.5 * z * erfc(-z / np.sqrt(2.0))
    return np.abs(e - 0.5 * erfc(a / np.sqrt(2.0))).max(), np.abs(gelu - exact).max()


if __name__ == "__main__":
    coef = fit()
    err_e, err_g = check(coef)
    print(f"// degree {DEGREE}: max |e - Phi(-a)| = {err_e:.2e}, max |GELU error| on [-12, 12] = {err_g:.2e}")
    print("constexpr float kGeluPoly[%d] = {" % (DEGREE + 1))
    print(",\n".join("    %.9ef" % x for x in coef) + "};")
    print("constexpr float kGeluClamp = %.9ef;" % f32(A))
