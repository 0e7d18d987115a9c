"""pow(a, b), atan2(a, b) and hypot(a, b) on the GPU through the expression paths.

NT2 policy: bit-identical to the oracle's restatement of NT2's float pow
(Cephes powf with NT2's special cases).  Fast policy: the float-float
log2/exp2 core, within 1.5 ulp of FP64 pow on finite results, including
results near overflow and in the subnormal range; special values as NT2.
"""
import json
import os

import numpy as np
import pytest
import torch

from helpers import nt2_ulpdist
from nt2_gb300 import expr as E
from nt2_gb300 import lib as L

pytestmark = pytest.mark.gpu
MODES = pytest.mark.parametrize("mode", [1, 2], ids=["compiled", "interpreter"])


def _pow(dev, x, y, prec, mode):
    tx, ty = torch.from_numpy(x).to(dev), torch.from_numpy(y).to(dev)
    out = torch.empty_like(tx)
    E.assign([out], [E.pow(E.Table(tx), E.Table(ty))], precision=prec, force_generic=mode)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _cases(n, seed):
    rng = np.random.default_rng(seed)
    xs, ys = [], []
    # wide magnitudes, moderate exponents
    xs.append(np.exp(rng.uniform(-80, 80, n))); ys.append(rng.uniform(-6, 6, n))
    # near 1 with large exponents
    xs.append(1 + rng.uniform(-1e-3, 1e-3, n)); ys.append(rng.uniform(-1e5, 1e5, n))
    # results near overflow and in the subnormal range
    b = np.exp(rng.uniform(0.1, 10, n))
    xs.append(b); ys.append((127 + rng.uniform(0, 0.999, n)) * np.log(2) / np.log(b))
    xs.append(b); ys.append(-(126 + rng.uniform(0, 23, n)) * np.log(2) / np.log(b))
    # negative bases with integer exponents (sign), and non-integer (NaN)
    xs.append(-np.exp(rng.uniform(-5, 5, n))); ys.append(rng.integers(-20, 20, n).astype(np.float64))
    xs.append(-np.exp(rng.uniform(-5, 5, n))); ys.append(rng.uniform(-3, 3, n))
    # subnormal bases
    xs.append(rng.uniform(0, 1.17e-38, n)); ys.append(rng.uniform(-0.5, 0.5, n))
    return np.concatenate(xs).astype(np.float32), np.concatenate(ys).astype(np.float32)


SPECIAL = np.array([0.0, -0.0, 1.0, -1.0, 2.0, -2.0, 0.5, np.inf, -np.inf, np.nan, 1e-45, 3e38], np.float32)


def _special_grid():
    a, b = np.meshgrid(SPECIAL, np.concatenate([SPECIAL, np.float32([3.0, -3.0, 0.25])]))
    return a.ravel().astype(np.float32), b.ravel().astype(np.float32)


@MODES
def test_pow_nt2_policy_bit_exact(dev, oracle, mode):
    x, y = _cases(1 << 16, 51)
    sx, sy = _special_grid()
    x, y = np.concatenate([x, sx]), np.concatenate([y, sy])
    got = _pow(dev, x, y, L.PREC_NT2, mode)
    ref = oracle.pow_f32(x, y)
    same = (got.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(got) & np.isnan(ref))
    assert same.all(), (x[~same][:4], y[~same][:4], got[~same][:4], ref[~same][:4])


@MODES
def test_pow_fast_policy_accuracy(dev, oracle, mode):
    x, y = _cases(1 << 17, 52)
    got = _pow(dev, x, y, L.PREC_FAST, mode)
    ref = oracle.pow_f64(x, y)
    fin = np.isfinite(ref) & (np.abs(ref) < 3.4e38) & (ref != 0)
    rf = np.abs(ref[fin]).astype(np.float32)
    ulp = np.where(rf < 1.1754944e-38, 1.4e-45, np.spacing(rf)).astype(np.float64)
    e = np.abs(got[fin].astype(np.float64) - ref[fin]) / ulp
    print(f"\npow fast policy vs FP64: max {e.max():.3f} mean {e.mean():.4f} ulp over {fin.sum()} points")
    assert e.max() <= 1.5, (x[fin][np.argmax(e)], y[fin][np.argmax(e)])
    # NaN exactly where FP64 pow is NaN (negative base, non-integer exponent)
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    # the special-value grid is NT2's, except where NT2's 16*b overflows
    # (|b| >= 2^124: NT2 returns NaN) and the fast policy returns FP64's value
    sx, sy = _special_grid()
    g, r = _pow(dev, sx, sy, L.PREC_FAST, mode), oracle.pow_f32(sx, sy)
    huge = np.abs(sy) >= 2.0 ** 124
    exact = (~np.isfinite(r) | (r == 0) | (np.abs(r) == 1)) & ~np.isnan(r) & ~huge
    assert np.array_equal(np.isnan(g[~huge]), np.isnan(r[~huge])) and np.array_equal(g[exact], r[exact])
    h = huge & np.isfinite(sy) & (sx > 0) & np.isfinite(sx) & (sx != 1)
    assert np.array_equal(g[h], oracle.pow_f64(sx[h], sy[h]).astype(np.float32))


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
def test_pow_golden_values(dev, prec):
    golden = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "nt2_unit_vectors.json")))
    recs = [r for r in golden if r["fn"] == "pow"]
    assert len(recs) == 10
    x = np.float32([r["x"] for r in recs])
    y = np.float32([r["y"] for r in recs])
    got = _pow(dev, x, y, prec, 1)
    for g, r in zip(got, recs):
        assert nt2_ulpdist(g, r["expected"]) <= r["tol_nt2ulp"], (r, g)
    recs = [r for r in golden if r["fn"] == "hypot"]
    assert len(recs) == 10
    hx, hy = torch.from_numpy(np.float32([r["x"] for r in recs])).to(dev), torch.from_numpy(np.float32([r["y"] for r in recs])).to(dev)
    ho = torch.empty_like(hx)
    E.assign([ho], [E.hypot(E.Table(hx), E.Table(hy))], precision=prec, force_generic=1)
    for g, r in zip(ho.cpu().numpy(), recs):
        assert nt2_ulpdist(g, r["expected"]) <= r["tol_nt2ulp"], (r, g)
    recs = [r for r in golden if r["fn"] == "atan2"]
    assert len(recs) == 14
    got = _atan2(dev, np.float32([r["x"] for r in recs]), np.float32([r["y"] for r in recs]), prec, 1)
    for g, r in zip(got, recs):
        assert nt2_ulpdist(g, r["expected"]) <= r["tol_nt2ulp"], (r, g)


def _atan2(dev, x, y, prec, mode):
    tx, ty = torch.from_numpy(x).to(dev), torch.from_numpy(y).to(dev)
    out = torch.empty_like(tx)
    E.assign([out], [E.atan2(E.Table(tx), E.Table(ty))], precision=prec, force_generic=mode)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@MODES
def test_atan2_both_policies(dev, oracle, mode):
    """atan2: NT2 policy bit-identical to the oracle, fast within 3 ulp of
    FP64, NT2's conventions at zeros and infinities in both."""
    rng = np.random.default_rng(53)
    n = 1 << 18
    x = (rng.standard_normal(n) * np.exp2(rng.integers(-20, 20, n))).astype(np.float32)
    y = (rng.standard_normal(n) * np.exp2(rng.integers(-20, 20, n))).astype(np.float32)
    sx, sy = _special_grid()
    x, y = np.concatenate([x, sx, sy]), np.concatenate([y, sy, sx])
    got = _atan2(dev, x, y, L.PREC_NT2, mode)
    ref = oracle.atan2_f32(x, y)
    assert np.all((got.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(got) & np.isnan(ref)))
    fast = _atan2(dev, x, y, L.PREC_FAST, mode)
    r64 = oracle.atan2_f64(x, y)
    m = np.isfinite(r64) & (np.abs(r64) > 1.2e-38) & (x != 0)
    e = np.abs(fast[m].astype(np.float64) - r64[m]) / np.spacing(np.abs(r64[m]).astype(np.float32))
    assert e.max() <= 3.0, float(e.max())
    z = (x == 0) | np.isnan(x) | np.isnan(y)
    assert np.all((fast[z].view(np.uint32) == ref[z].view(np.uint32)) | (np.isnan(fast[z]) & np.isnan(ref[z])))


@MODES
def test_hypot_both_policies(dev, oracle, mode):
    """hypot: NT2 policy bit-identical to the oracle (NT2's scaled form), fast
    within 1.5 ulp of FP64, no overflow or underflow in the intermediates,
    inf when one operand is NaN and the other infinite."""
    rng = np.random.default_rng(54)
    n = 1 << 18
    x = (rng.uniform(-2, 2, n) * np.exp2(rng.integers(-149, 127, n))).astype(np.float32)
    y = (rng.uniform(-2, 2, n) * np.exp2(rng.integers(-149, 127, n))).astype(np.float32)
    sx, sy = _special_grid()
    x, y = np.concatenate([x, sx, sy]), np.concatenate([y, sy, sx])
    tx, ty = torch.from_numpy(x).to(dev), torch.from_numpy(y).to(dev)
    for prec in (L.PREC_NT2, L.PREC_FAST):
        out = torch.empty_like(tx)
        E.assign([out], [E.hypot(E.Table(tx), E.Table(ty))], precision=prec, force_generic=mode)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        if prec == L.PREC_NT2:
            ref = oracle.hypot_f32(x, y)
            assert np.all((got.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(got) & np.isnan(ref)))
        else:
            r64 = oracle.hypot_f64(x, y)
            fin = np.isfinite(r64) & (r64 < 3.4e38)
            rf = r64[fin].astype(np.float32)
            ulp = np.where(rf < 1.1754944e-38, 1.4e-45, np.spacing(rf)).astype(np.float64)
            assert (np.abs(got[fin] - r64[fin]) / ulp).max() <= 1.5
            assert np.array_equal(np.isnan(got), np.isnan(r64) & ~np.isinf(x) & ~np.isinf(y))
