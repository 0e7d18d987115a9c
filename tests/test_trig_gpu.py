"""sin, cos, tan, sinpi, cospi, cot, sec, csc, sind, cosd, tand on the GPU.

NT2 policy: bit-identical to the oracle's restatement of NT2's float
algorithms (trig_base.hpp with its reduction cascade: straight, Cody-Waite,
the compensated three-step form in float and in double, and the exact
reduction beyond 2^18 pi).  Fast policy: within 2 ulp of FP64 for sin, cos,
sinpi, cospi and 3.5 ulp for tan over every reduction band, special values as
NT2 has them (sinpi/cospi of |x| >= 2^127 excepted: NT2's 2x overflows to a
NaN there, the fast policy returns the exact +-0 / 1).  cot, sec and csc
(radian reduction, then NT2's cotangent branch or a division) within 3.5 ulp for cot, 3 for sec and csc;
the degree functions (round(x/90) reduction) within 1.75 ulp for sind/cosd
and 3 for tand while the float remainder x - 90 k is exact (|x| <= 1e6).
"""
import json
import os

import numpy as np
import pytest
import torch

from helpers import nt2_ulpdist, std_ulp

pytestmark = pytest.mark.gpu

FNS = ["sin", "cos", "tan", "sinpi", "cospi"]
MORE = ["cot", "sec", "csc", "sind", "cosd", "tand"]
DEGREES = ("sind", "cosd", "tand")
FAST_TOL = dict(sin=2.0, cos=2.0, tan=3.5, sinpi=2.0, cospi=2.0, cot=3.5, sec=3.0, csc=3.0, sind=1.75, cosd=1.75,
                tand=3.0)
SPECIALS = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, -1e-45, 1e-40, 0.5, -0.5, 0.25, 1.0, -1.0,
                     0.785398185, 0.785398245, 1.57079637, 1.5707965, 62.8318520, 62.8318558, 201.061920,
                     201.061951, 823549.5625, 823549.625, 823549.6875, 823549.75, 131072.0, 131072.02,
                     8388608.0, 8388609.0, 16777216.0, 1e20, 1.7e38, 3.4e38, -3.4e38, 2.0 ** 127],
                    np.float32)


def _bands(n, seed):
    rng = np.random.default_rng(seed)
    parts = [rng.uniform(-1, 1, n), rng.uniform(-1.6, 1.6, n), rng.uniform(-63, 63, n), rng.uniform(-201, 201, n),
             rng.uniform(-1.4e5, 1.4e5, n), rng.uniform(-8.3e5, 8.3e5, n),
             np.exp(rng.uniform(np.log(8e5), np.log(3.4e38), n)) * rng.choice([-1, 1], n)]
    return np.concatenate(parts).astype(np.float32)


def _degree_bands(n, seed):
    rng = np.random.default_rng(seed)
    parts = [rng.uniform(-90, 90, n), rng.uniform(-720, 720, n), rng.uniform(-1e6, 1e6, n),
             rng.integers(-8000, 8000, n) * 45.0, rng.integers(-2000, 2000, n) * 30.0]
    return np.concatenate(parts).astype(np.float32)


def _gpu(lib, dev, fn, x, prec):
    tx = torch.from_numpy(x).to(dev)
    ty = torch.empty_like(tx)
    lib.map_f32(fn, tx, ty, precision=prec)
    torch.cuda.synchronize()
    return ty.cpu().numpy()


def _same(a, b):
    return (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))


@pytest.mark.parametrize("fn", FNS + MORE)
def test_trig_nt2_policy_bit_exact(lib, dev, oracle, fn):
    x = np.concatenate([_bands(1 << 19, 41), SPECIALS, -SPECIALS])
    if fn in DEGREES:
        x = np.concatenate([x, _degree_bands(1 << 18, 43)])
    got = _gpu(lib, dev, fn, x, lib.PREC_NT2)
    ref = oracle.map_f32(fn, x)
    same = _same(got, ref)
    assert same.all(), f"{(~same).sum()} differ, first at x={x[~same][:5]} got {got[~same][:5]} want {ref[~same][:5]}"


@pytest.mark.parametrize("fn", FNS + MORE)
def test_trig_fast_policy_accuracy(lib, dev, oracle, fn):
    x = _degree_bands(1 << 19, 42) if fn in DEGREES else _bands(1 << 19, 42)
    got = _gpu(lib, dev, fn, x, lib.PREC_FAST)
    ref = oracle.map_f64(fn, x)
    m = np.isfinite(ref) & (np.abs(ref) >= np.finfo(np.float32).tiny) & (np.abs(ref) < 3e38)
    if fn == "tand":  # NT2's singularity test, (x - 90)/180 integral in float, holds in both policies
        nt2nan = np.isnan(oracle.map_f32(fn, x))
        assert np.isnan(got[nt2nan]).all()
        m &= ~nt2nan
    e = std_ulp(got[m], ref[m])
    print(f"\n{fn}: fast policy vs FP64 max {e.max():.3f} mean {e.mean():.4f} ulp over {m.sum()} points")
    assert e.max() <= FAST_TOL[fn], f"max {e.max()} ulp at x={x[m][np.argmax(e)]}"
    # exact zeros of sinpi/cospi stay exact zeros
    z = ~m & np.isfinite(x) & (ref == 0)
    assert (got[z] == 0).all()


def test_trig_fast_strided_all_floats(lib, dev, oracle):
    """Every 61st positive float (all exponents, all reduction bands) for sin,
    cos and tan against FP64."""
    bits = np.arange(0, 0x7f800000, 61, dtype=np.uint32)
    x = bits.view(np.float32)
    for fn in ("sin", "cos", "tan"):
        got = _gpu(lib, dev, fn, x, lib.PREC_FAST)
        ref = oracle.map_f64(fn, x)
        m = (np.abs(ref) >= np.finfo(np.float32).tiny) & (np.abs(ref) < 3e38)
        e = std_ulp(got[m], ref[m])
        assert e.max() <= FAST_TOL[fn], (fn, float(e.max()), x[m][np.argmax(e)])
        sub = ~m & (np.abs(ref) < 3e38)  # subnormal results: sin x = tan x = x there
        assert (np.abs(got[sub].astype(np.float64) - ref[sub]) <= 1.5e-45).all()


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
def test_trig_specials(lib, dev, prec):
    x = np.float32([0.0, -0.0, np.inf, -np.inf, np.nan])
    for fn in FNS:
        got = _gpu(lib, dev, fn, x, prec)
        assert np.isnan(got[2:]).all(), fn
        if fn in ("sin", "tan", "sinpi"):
            assert got[0] == 0 and not np.signbit(got[0]) and got[1] == 0 and np.signbit(got[1]), fn
        else:
            assert (got[:2] == 1).all(), fn
    big = np.float32([2.0 ** 127, 3.4e38, -3.4e38])
    if prec == 0:
        assert np.array_equal(_gpu(lib, dev, "cospi", big, prec), [1, 1, 1])
        assert np.array_equal(_gpu(lib, dev, "sinpi", big, prec), [0, 0, 0])
    else:
        assert np.isnan(_gpu(lib, dev, "cospi", big, prec)).all()
    want = dict(cot=[np.inf, -np.inf], sec=[1, 1], csc=[np.inf, -np.inf], sind=[0.0, -0.0], cosd=[1, 1],
                tand=[0.0, -0.0])
    for fn in MORE:
        got = _gpu(lib, dev, fn, x, prec)
        assert np.isnan(got[2:]).all(), fn
        assert np.array_equal(got[:2], np.float32(want[fn])) and np.array_equal(np.signbit(got[:2]),
                                                                                 np.signbit(want[fn])), fn
    quarter = np.float32([90, -90, 270, 180, -180, 45, -45, 30, 60])
    assert np.isnan(_gpu(lib, dev, "tand", quarter, prec)[:3]).all()
    assert np.array_equal(_gpu(lib, dev, "cosd", quarter[:2], prec), [0, 0])
    assert np.array_equal(_gpu(lib, dev, "sind", quarter[:2], prec), [1, -1])


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
def test_trig_golden_values(lib, dev, prec):
    golden = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "nt2_unit_vectors.json")))
    recs = [r for r in golden if r["fn"] in FNS + MORE]
    assert len(recs) >= 96
    for rec in recs:
        got = _gpu(lib, dev, rec["fn"], np.array([rec["x"]], np.float32), prec)[0]
        assert nt2_ulpdist(got, rec["expected"]) <= rec["tol_nt2ulp"], (rec, got)
