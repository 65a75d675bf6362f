"""Derives the polynomial coefficients used by gls_clmath.h.

Each approximation is a weighted least-squares fit on Chebyshev nodes,
refined by Lawson's iteratively reweighted least squares towards the
minimax (equi-ripple) relative-error solution.  Run it with numpy to
reproduce the constants printed into gls_clmath.h:

    python climage_gb300/csrc/fit_clmath_coeffs.py
"""
import numpy as np


def lawson_fit(f, lo, hi, basis, n_nodes=4000, iters=60, rel=True):
    k = np.arange(n_nodes)
    t = np.cos((2 * k + 1) * np.pi / (2 * n_nodes))
    x = 0.5 * (lo + hi) + 0.5 * (hi - lo) * t
    y = f(x)
    A = np.stack([b(x) for b in basis], axis=1)
    scale = np.abs(y) if rel else np.ones_like(y)
    scale[scale == 0] = 1
    w = np.ones_like(x) / n_nodes
    coef = None
    for _ in range(iters):
        sw = np.sqrt(w)
        coef, *_ = np.linalg.lstsq(A * (sw / scale)[:, None], y * sw / scale, rcond=None)
        err = np.abs(A @ coef - y) / scale
        w = w * err
        w = w / w.sum()
    err = np.abs(A @ coef - y) / scale
    return coef, err.max()


def main():
    # atan(a) / (pi * a) as a polynomial in s = a^2 on [0, 1]
    deg = 9
    f = lambda s: np.where(s > 0, np.arctan(np.sqrt(s)) / (np.pi * np.sqrt(np.maximum(s, 1e-300))), 1 / np.pi)
    c, e = lawson_fit(f, 0.0, 1.0, [lambda s, i=i: s ** i for i in range(deg + 1)])
    print("atan/pi coeffs (s^0..):", ", ".join("%.9e" % v for v in c), "max rel err %.3e" % e)

    # (tanh(x) / x - 1) / x^2 as a polynomial in s = x^2 on [0, 0.625^2]
    deg = 6
    f = lambda s: (np.tanh(np.sqrt(s)) / np.sqrt(s) - 1) / s
    c, e = lawson_fit(f, 1e-8, 0.625 ** 2, [lambda s, i=i: s ** i for i in range(deg + 1)])
    print("tanh coeffs (s^0..):", ", ".join("%.9e" % v for v in c), "max rel err %.3e" % e)

    # 2^f on [-0.5, 0.5]
    deg = 6
    c, e = lawson_fit(lambda x: 2.0 ** x, -0.5, 0.5, [lambda x, i=i: x ** i for i in range(deg + 1)])
    print("exp2 coeffs (f^0..):", ", ".join("%.9e" % v for v in c), "max rel err %.3e" % e)

    # log2(m) = z * P(z^2), z = (m - 1) / (m + 1), m in [sqrt(1/2), sqrt(2)]
    zmax = (np.sqrt(2) - 1) / (np.sqrt(2) + 1)
    deg = 5
    f = lambda s: np.log2((1 + np.sqrt(s)) / (1 - np.sqrt(s))) / np.sqrt(s)
    c, e = lawson_fit(f, 1e-10, zmax ** 2, [lambda s, i=i: s ** i for i in range(deg + 1)])
    print("log2 coeffs (z2^0..):", ", ".join("%.9e" % v for v in c), "max rel err %.3e" % e)


if __name__ == "__main__":
    main()
