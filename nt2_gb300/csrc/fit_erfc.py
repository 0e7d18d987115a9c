"""Derive the erfc tail polynomial used by the fast device math (nt2g_math.cuh).

Method (published form, own coefficients): for t >= 0,

    erfc(t) = exp(-t^2) * w * R(w),   w = 1 / (1 + p*t),  p = 1/2

with R evaluated as a polynomial in d = w - 1/2 (|d| <= 1/2 keeps the
float32 Horner rounding small),

which is the parametrisation of the Chebyshev-fitted erfc in Press et al.,
Numerical Recipes (2nd ed.), section 6.2, with the polynomial kept as a
multiplier instead of inside the exponent.  R(w) = erfcx(t)/w is smooth on
w in (0, 1], so one branch-free polynomial covers the whole half-line.  The
coefficients are a relative-error fit on Chebyshev nodes driven towards
minimax by Lawson's iteratively reweighted least squares, rounded to float32
one coefficient at a time from the highest degree down (re-fitting the rest
after each rounding), and finally polished by a small search over +-2 ulp of
the three lowest-degree coefficients.

Run:  python nt2_gb300/csrc/fit_erfc.py   (needs numpy and scipy)
It prints the coefficients (highest degree first, as C hex-float literals)
and the maximum relative error of the float32 polynomial in ulp.
"""
import numpy as np
from scipy.special import erfcx

P = 0.5
DEG = 10
CENTER = 0.5


def _nodes(m=6000):
    k = np.arange(m)
    w = 0.5 * (1.0 - np.cos(np.pi * (k + 0.5) / m))
    return np.clip(w, 1e-9, 1.0)


def _target(w):
    t = (1.0 - w) / (w * P)
    return erfcx(t) / w


def _lawson(w, y, r, deg, iters=60):
    """Weighted LSQ of y ~ poly(w) (relative to r), reweighted towards minimax."""
    wt = np.ones_like(w)
    for _ in range(iters):
        c = np.polynomial.polynomial.polyfit(w, y, deg, w=np.sqrt(wt) / np.abs(r))
        err = np.abs((np.polynomial.polynomial.polyval(w, c) - y) / r)
        wt = wt * (err + 1e-300)
        wt /= wt.sum()
    return c


def _horner32(coeffs, w):
    acc = np.full_like(w, np.float32(coeffs[0]), dtype=np.float32)
    w32 = (w.astype(np.float32) - np.float32(CENTER)).astype(np.float32)
    for c in coeffs[1:]:
        acc = (acc.astype(np.float64) * w32 + np.float64(np.float32(c))).astype(np.float32)
    return acc.astype(np.float64)


def fit():
    w = _nodes()
    r = _target(w)
    d = w - CENTER
    fixed = []  # float32-rounded coefficients, highest degree first
    for deg in range(DEG, -1, -1):
        # remove the contribution of the already rounded higher-degree terms
        resid = r.copy()
        for j, c in enumerate(fixed):
            resid -= float(c) * d ** (DEG - j)
        c = _lawson(d, resid, r, deg)
        fixed.append(np.float32(c[deg]))
    # polish: +-2 ulp on the three lowest-degree coefficients, scored on the
    # float32 Horner evaluation
    ws = np.linspace(1e-7, 1.0, 100001)
    rs = _target(ws)
    best = (np.max(np.abs(_horner32(fixed, ws) / rs - 1.0)), list(fixed))
    for i in range(DEG - 2, DEG + 1):
        for _pass in range(2):
            base = list(best[1])
            for k in range(-2, 3):
                cand = list(base)
                cand[i] = np.float32(np.nextafter(np.float32(base[i]), np.float32(np.inf * np.sign(k)))) if k else base[i]
                for _ in range(abs(k) - 1):
                    cand[i] = np.float32(np.nextafter(cand[i], np.float32(np.inf * np.sign(k))))
                e = np.max(np.abs(_horner32(cand, ws) / rs - 1.0))
                if e < best[0]:
                    best = (e, cand)
    return best[1]


def max_ulp(coeffs):
    """Max relative error of the float32 Horner evaluation, in units of 2^-24."""
    w = np.linspace(1e-7, 1.0, 400001)
    return np.max(np.abs(_horner32(coeffs, w) / _target(w) - 1.0)) / 2.0 ** -24


if __name__ == "__main__":
    cs = fit()
    for c in cs:
        print(f"{float(c).hex()}f,  /* {float(c): .9e} */")
    print("max rel error of the float32 polynomial: %.3f ulp" % max_ulp(cs))
