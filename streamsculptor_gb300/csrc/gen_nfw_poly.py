"""Fit the polynomial of the FP32 NFW enclosed-mass function (nfw_F2 in
ss_stream2.cuh) and report its accuracy.

NFW's F(u) = ln(1+u) - u/(1+u) is written for u < 2, with s = u / (2+u) and
w = s^2 <= 1/4, as F = s (u / (1+u) + w P(w)), where
P(w) = 2 sum_k w^k / (2k+3) (from ln(1+u) = 2 atanh(s)).  P is fitted by a
polynomial of degree 6 in w, least squares in relative error at 4000
Chebyshev nodes of [0, 1/4]; the kernel uses the coefficients rounded to
FP32.  The script prints them, the fit's relative error with the rounded
coefficients, and the error of F evaluated with FP32 rounding after every
operation (the kernel's sequence, the reciprocal modelled as correctly
rounded before its Newton step) against the FP64 value, over u in (0, 2).

Run: python gen_nfw_poly.py
"""
import numpy as np

DEG = 6


def fit(deg: int = DEG) -> np.ndarray:
    w = np.cos(np.pi * (np.arange(4000) + 0.5) / 4000) * 0.125 + 0.125
    p = 2.0 * sum(w**k / (2 * k + 3) for k in range(40))
    a = np.vstack([w**k for k in range(deg + 1)]).T
    c = np.linalg.lstsq(a / p[:, None], np.ones_like(w), rcond=None)[0]
    c32 = c.astype(np.float32)
    err = np.max(np.abs(a @ c32.astype(np.float64) - p) / p)
    return c32, err


def _r(x):
    return np.asarray(x, dtype=np.float64).astype(np.float32)


def f32_F(u: np.ndarray, c: np.ndarray) -> np.ndarray:
    """F(u) with FP32 rounding after each operation, as nfw_F2 orders them."""
    fma = lambda a, b, d: _r(np.float64(a) * np.float64(b) + np.float64(d))
    mul = lambda a, b: _r(np.float64(a) * np.float64(b))
    add = lambda a, b: _r(np.float64(a) + np.float64(b))

    def rcp(x):
        r = _r(1.0 / np.float64(x))
        e = fma(x, r, np.float32(-1))
        return fma(-r, e, r)

    A, B = add(np.float32(2), u), add(np.float32(1), u)
    uR = mul(u, rcp(mul(A, B)))
    s = mul(uR, B)
    w = mul(s, s)
    P = fma(c[DEG], w, c[DEG - 1])
    for k in range(DEG - 2, -1, -1):
        P = fma(P, w, c[k])
    return mul(s, fma(w, P, mul(uR, A)))


def main():
    c, err = fit()
    print("coefficients c_0 .. c_%d:" % DEG, ", ".join("%.9gf" % x for x in c))
    print("fit relative error (FP32 coefficients): %.2e" % err)
    u = np.concatenate([np.geomspace(1e-6, 1e-4, 2000), np.linspace(1e-4, 2, 200001)]).astype(np.float32)
    U = u.astype(np.float64)
    ref = np.log1p(U) - U / (1 + U)
    rel = np.abs(f32_F(u, c) - ref) / ref
    print("F in FP32 over u in (0, 2): max %.2e, median %.2e relative" % (rel.max(), np.median(rel)))


if __name__ == "__main__":
    main()
