"""Fits the arctangent polynomial used by trax_math.h.

Method: atan(t) on [0, 1] is written as t + t^3 * P(t^2), with P of degree 8
(nine coefficients). P is fitted to minimise the maximum *relative* error of
atan over a dense grid, by Lawson's iteratively reweighted least squares (the
weights converge to the Chebyshev/minimax solution).  The coefficients are then
rounded to float32 and the float32 Horner evaluation is checked against
double-precision arctan.

Run `python fit_atan.py` to reprint the table embedded in trax_math.h.
"""
import numpy as np

NTERMS = 9


def fit(nterms=NTERMS, iters=60):
    t = np.cos(np.linspace(0.0, np.pi / 2, 20000))
    t = np.unique(np.concatenate([t, np.linspace(1e-4, 1.0, 20000)]))
    s = t * t
    target = (np.arctan(t) - t) / (t ** 3)
    a = np.vstack([s ** k for k in range(nterms)]).T
    w = np.ones_like(t)
    for _ in range(iters):
        sw = np.sqrt(w)
        c, *_ = np.linalg.lstsq(a * sw[:, None], target * sw, rcond=None)
        err = np.abs(t + t ** 3 * (a @ c) - np.arctan(t)) / np.arctan(t)
        w = w * err
        w /= w.sum()
    return c.astype(np.float32)


def eval_f32(c, t):
    """Float32 evaluation with exactly the operation order of trax_atan01."""
    t = t.astype(np.float32)
    s = (t * t).astype(np.float32)
    p = c[-1]
    for k in range(len(c) - 2, -1, -1):
        p = (p * s).astype(np.float32)
        p = (p + c[k]).astype(np.float32)
    r = (t * s).astype(np.float32)
    r = (r * p).astype(np.float32)
    return (t + r).astype(np.float32)


def max_ulp(c, n=2_000_000, seed=0):
    t = np.random.default_rng(seed).random(n).astype(np.float32)
    ref = np.arctan(t.astype(np.float64))
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    return float(np.max(np.abs(eval_f32(c, t).astype(np.float64) - ref) / ulp))


if __name__ == "__main__":
    c = fit()
    for k, v in enumerate(c):
        print(f"    {float(v).hex()}f, /* c{k} = {float(v):.9e} */")
    print("max ulp on [0,1]:", max_ulp(c))
