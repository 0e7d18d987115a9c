"""Regenerate gammainc_large_a.json: reference values of the regularised
lower incomplete gamma function P(a, x) for large a, where scipy's double
gammainc is not accurate enough to check a float result (at a = 1e8,
x = 0.999 a it is 15% off).

Evaluated in 50-digit arithmetic (mpmath) by the defining series
P = x^a e^-x / Gamma(a+1) sum_k x^k / ((a+1)...(a+k)) for x <= a, and by
Legendre's continued fraction for Q = 1 - P above (modified Lentz), each
summed until its terms fall below 1e-30 of the total.  Inputs are float32
values (as the GPU receives them); the outputs are doubles.

Usage:  python tests/golden/make_gammainc.py
"""
import json
import os

import mpmath as mp
import numpy as np

mp.mp.dps = 50


def p_series(a, x):
    t = s = mp.mpf(1)
    k = 0
    while True:
        k += 1
        t *= x / (a + k)
        s += t
        if t < s * mp.mpf(10) ** -30:
            break
    return mp.exp(a * mp.log(x) - x - mp.loggamma(a + 1)) * s


def q_fraction(a, x):
    tiny = mp.mpf(10) ** -60
    b = x + 1 - a
    c, d = 1 / tiny, 1 / b
    h = d
    i = 0
    while True:
        i += 1
        an = -i * (i - a)
        b += 2
        d = an * d + b
        d = tiny if abs(d) < tiny else d
        c = b + an / c
        c = tiny if abs(c) < tiny else c
        d = 1 / d
        delta = d * c
        h *= delta
        if abs(delta - 1) < mp.mpf(10) ** -30:
            break
    return mp.exp(a * mp.log(x) - x - mp.loggamma(a)) * h


def main():
    out = []
    for a in (2e5, 9.9e5, 1.01e6, 4e6, 1e7, 1e8, 1e9):
        af = float(np.float32(a))
        for r in (0.99, 0.995, 0.999, 0.9995, 1.0, 1.0005, 1.001, 1.005, 1.01):
            xf = float(np.float32(np.float32(af) * np.float32(r)))
            A, X = mp.mpf(af), mp.mpf(xf)
            p = p_series(A, X) if X <= A else 1 - q_fraction(A, X)
            out.append(dict(a=af, x=xf, p=float(p)))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "gammainc_large_a.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {len(out)} records to {path}")


if __name__ == "__main__":
    main()
