"""NT2's exact arithmetic functors on the GPU: floor, ceil, trunc (fix), round,
round2even, frac, sign, signnz, copysign, mod, rem, pow2 and the compositions oneplus,
oneminus, minusone, sqr_abs, dist, average (boost/simd arithmetic and ieee
functors).  Each is correctly rounded (or exact), so both policies must equal
the oracle bit for bit -- average excepted under the fast policy, whose fma is
fused (within half an ulp there).  Known answers: the float cases of
boost.simd's own unit tests.
"""
import json
import math
import os

import numpy as np
import pytest
import torch

from helpers import nt2_ulpdist

pytestmark = pytest.mark.gpu

UNARY = ["floor", "ceil", "trunc", "fix", "round", "round2even", "frac", "sign", "signnz", "oneplus", "oneminus",
         "minusone", "sqr_abs"]
BINARY = ["copysign", "dist", "average", "mod", "rem", "pow2", "maxnum", "minnum", "maxmag", "minmag", "minmod",
          "negate", "divfloor", "divceil", "divfix", "divround", "divround2even"]
NT2_NAN = float(np.uint32(0xffffffff).view(np.float32))  # NT2's Nan<T>(): every bit set


def _inputs(seed, n=1 << 13):
    rng = np.random.default_rng(seed)
    sp = np.float32([0.0, -0.0, np.inf, -np.inf, np.nan, NT2_NAN, 0.5, -0.5, 1.5, -1.5, 2.5, -2.5, 0.49999997,
                     -0.49999997, 8388607.5, 8388608.0, -8388607.5, 16777216.0, 1e-45, -1e-45, 3.4e38, -3.4e38])
    x = np.concatenate([rng.uniform(-10, 10, n), rng.integers(-20, 20, n) * 0.5,
                        np.exp(rng.uniform(-100, 88, n)) * rng.choice([-1.0, 1.0], n)]).astype(np.float32)
    return np.concatenate([x, sp])


def _same(a, b):
    return (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))


def _eval(dev, expr_of, xs, prec):
    from nt2_gb300 import expr as E
    ts = [torch.from_numpy(x).to(dev) for x in xs]
    out = torch.empty_like(ts[0])
    E.assign([out], [expr_of(E, *[E.Table(t) for t in ts])], precision=prec)
    return out.cpu().numpy()


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
@pytest.mark.parametrize("fn", UNARY)
def test_unary_bit_exact(lib, dev, oracle, fn, prec):
    x = _inputs(21)
    got = _eval(dev, lambda E, a: getattr(E, fn)(a), [x], prec)
    f = getattr(oracle.lib(), "o_" + fn)
    want = np.float32([f(float(v)) for v in x])
    same = _same(got, want)
    assert same.all(), (x[~same][:5], got[~same][:5], want[~same][:5])
    if fn in ("sign", "signnz"):  # NaN stays NaN; the rest is exactly -1, 0 or 1
        assert set(np.unique(got[~np.isnan(got)])) <= {-1.0, 0.0, 1.0}


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
@pytest.mark.parametrize("fn", BINARY)
def test_binary(lib, dev, oracle, fn, prec):
    a, b = _inputs(22), _inputs(23)[::-1].copy()
    got = _eval(dev, lambda E, p, q: getattr(E, fn)(p, q), [a, b], prec)
    f = getattr(oracle.lib(), "o_" + fn)
    want = np.float32([f(float(p), float(q)) for p, q in zip(a, b)])
    if fn == "average" and prec == 0:  # fused: within half an ulp of NT2's twice-rounded form
        with np.errstate(invalid="ignore"):
            ok = _same(got, want) | (np.abs(got.astype(np.float64) - want) <= np.spacing(np.abs(want)))
    else:
        ok = _same(got, want)
    assert ok.all(), (a[~ok][:5], b[~ok][:5], got[~ok][:5], want[~ok][:5])


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
def test_golden_values(lib, dev, prec):
    golden = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "nt2_unit_vectors.json")))
    arg = lambda v: NT2_NAN if math.isnan(v) else v
    recs = [r for r in golden if r["fn"] in UNARY + BINARY]
    assert len(recs) >= 100
    for r in recs:
        xs = [np.float32([arg(r["x"])])] + ([np.float32([arg(r["y"])])] if "y" in r else [])
        got = _eval(dev, lambda E, *t: getattr(E, r["fn"])(*t), xs, prec)[0]
        assert nt2_ulpdist(got, r["expected"]) <= r["tol_nt2ulp"], (r, got)


@pytest.mark.parametrize("mode", [0, 1, 2], ids=["fused-or-jit", "jit", "interp"])
def test_predicates(lib, dev, mode):
    """is_nan, is_inf, is_finite (NT2: x - x == 0), is_eqz, is_nez, is_ltz, is_gtz as logical values: selected
    by if_else and stored directly (0.0 / 1.0), identical in the compiled kernel and the interpreter."""
    from nt2_gb300 import expr as E
    x = _inputs(24)
    tx = torch.from_numpy(x).to(dev)
    names = ["is_nan", "is_inf", "is_finite", "is_eqz", "is_nez", "is_ltz", "is_gtz"]
    with np.errstate(invalid="ignore"):
        want = {"is_nan": np.isnan(x), "is_inf": np.isinf(x), "is_finite": np.isfinite(x), "is_eqz": x == 0,
                "is_nez": x != 0, "is_ltz": x < 0, "is_gtz": x > 0}
    outs = [torch.empty_like(tx) for _ in range(2 * len(names))]
    X = E.Table(tx)
    exprs = []
    for n in names:
        exprs += [E.if_else(getattr(E, n)(X), 2.0, -3.0), getattr(E, n)(X)]
    E.assign(outs, exprs, force_generic=mode)
    for k, n in enumerate(names):
        sel, raw = outs[2 * k].cpu().numpy(), outs[2 * k + 1].cpu().numpy()
        assert np.array_equal(sel, np.where(want[n], 2.0, -3.0).astype(np.float32)), n
        assert np.array_equal(raw, want[n].astype(np.float32)), n
