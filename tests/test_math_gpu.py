"""Element functions on the GPU: NT2 policy bit-identical to the oracle (the
CPU restatement of NT2's scalar algorithms); fast policy within 4 standard
ulp of FP64; both within NT2's own unit-test tolerances on its golden
values."""
import json
import os

import numpy as np
import pytest
import torch

from helpers import nt2_ulpdist, std_ulp

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "nt2_unit_vectors.json")))
SPECIALS = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, 1e-40, -1e-40, 1e-45, 3e38, -3e38, 0.5,
                     2 / 3, -2 / 3, 88.3763, -88.3763, 88.7, -103.0, 9.3, 13.2, -13.2, 0.6666666,
                     127.0, -127.0, 126.6, -126.6, 128.0, 38.23, -37.9, 38.5, -38.5, -15.9424, -15.95, -17.0],
                    np.float32)

# domain of each function for the accuracy sweep (finite FP64 reference above
# the float normal range)
DOMAINS = dict(exp=(-87.3, 88.3), log=(1e-30, 1e30), log1p=(-0.999, 1e4), erfc=(-10, 9.2), normcdf=(-13, 9),
               fastnormcdf=(-9, 9), sqrt=(0, 1e30), exp2=(-126, 126.99), exp10=(-37.8, 38.2),
               expm1=(-20, 88.37), log2=(1e-30, 1e30), log10=(1e-30, 1e30), sinh=(-89, 89), cosh=(-89, 89),
               tanh=(-12, 12), asin=(-1, 1), acos=(-1, 1), atan=(-1e4, 1e4), asinh=(-1e4, 1e4), acosh=(1, 1e4),
               atanh=(-0.9999999, 0.9999999), cbrt=(-1e30, 1e30))


def _sweep(fn, n=1 << 22, seed=5):
    lo, hi = DOMAINS[fn]
    rng = np.random.default_rng(seed)
    if fn in ("log", "log2", "log10", "sqrt"):
        x = np.concatenate([np.geomspace(max(lo, 1e-38), hi, n // 2), rng.uniform(0, 4, n // 2)])
    else:
        x = np.concatenate([np.linspace(lo, hi, n // 2), rng.uniform(lo, hi, n // 4),
                            rng.uniform(-1, 1, n // 4)])
    return x.astype(np.float32)


def _inputs(fn, n=1 << 22, seed=5):
    return np.concatenate([_sweep(fn, n, seed), SPECIALS])


def _gpu_map(lib, dev, fn, x, prec):
    tx = torch.from_numpy(x).to(dev)
    ty = torch.empty_like(tx)
    lib.map_f32(fn, tx, ty, precision=prec)
    torch.cuda.synchronize()
    return ty.cpu().numpy()


@pytest.mark.parametrize("fn", ["exp", "log", "log1p", "erfc", "normcdf", "fastnormcdf", "sqrt", "exp2", "exp10",
                                "expm1", "log2", "log10", "sinh", "cosh", "tanh", "asin", "acos", "atan",
                                "asinh", "acosh", "atanh", "cbrt"])
def test_nt2_policy_bit_exact(lib, dev, oracle, fn):
    x = _inputs(fn)
    got = _gpu_map(lib, dev, fn, x, lib.PREC_NT2)
    ref = oracle.map_f32(fn, x)
    same = (got.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(got) & np.isnan(ref))
    assert same.all(), f"{(~same).sum()} differ, first at x={x[~same][:5]}"


@pytest.mark.parametrize("fn,tol", [("exp", 1.5), ("log", 1.5), ("log1p", 2.0), ("erfc", 4.0), ("normcdf", 4.0),
                                    ("sqrt", 0.5), ("exp2", 2.0), ("exp10", 2.0), ("expm1", 2.0),
                                    ("log2", 1.5), ("log10", 1.5), ("sinh", 3.0), ("cosh", 3.0), ("tanh", 2.0),
                                    ("asin", 3.0), ("acos", 2.0), ("atan", 3.0), ("asinh", 2.5), ("acosh", 3.0),
                                    ("atanh", 3.0), ("cbrt", 2.0)])
def test_fast_policy_within_4ulp_of_fp64(lib, dev, oracle, fn, tol):
    """Accuracy over each function's sweep domain; the special values
    (including exp's +inf from NT2's Maxlog = 88.3763 on, as NT2) are
    checked against NT2's conventions separately."""
    x = _sweep(fn)
    got = _gpu_map(lib, dev, fn, x, lib.PREC_FAST)
    ref = oracle.map_f64(fn, x)
    m = np.isfinite(ref) & (np.abs(ref) >= np.finfo(np.float32).tiny)
    e = std_ulp(got[m], ref[m])
    print(f"\n{fn}: fast policy vs FP64 max {e.max():.3f} mean {e.mean():.4f} ulp over {m.sum()} points")
    assert e.max() <= tol, f"max {e.max()} ulp at x={x[m][np.argmax(e)]}"
    # specials agree with IEEE / NT2 conventions
    sp = _gpu_map(lib, dev, fn, SPECIALS, lib.PREC_FAST)
    ref_sp = oracle.map_f32(fn, SPECIALS)
    both_nan = np.isnan(sp) == np.isnan(ref_sp)
    assert both_nan.all()
    inf = np.isinf(ref_sp)
    assert np.array_equal(sp[inf], ref_sp[inf])


def test_fast_normcdf_pair_complement(lib, dev, oracle):
    x = _sweep("normcdf")
    neg = _gpu_map(lib, dev, "normcdf_neg", x, lib.PREC_FAST)  # normcdf(-x) from the shared core
    ref = oracle.map_f64("normcdf", -x)
    m = np.isfinite(ref) & (ref >= np.finfo(np.float32).tiny)
    assert std_ulp(neg[m], ref[m]).max() <= 4.0


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
def test_golden_values_on_gpu(lib, dev, prec):
    for rec in [r for r in GOLDEN if r["fn"] in ("exp", "log", "erfc", "normcdf", "fastnormcdf", "exp2", "exp10",
                                                  "expm1", "log2", "log10", "sinh", "cosh", "tanh", "asin",
                                                  "acos", "atan", "asinh", "acosh", "atanh", "cbrt")]:
        got = _gpu_map(lib, dev, rec["fn"], np.array([rec["x"]], np.float32), prec)[0]
        assert nt2_ulpdist(got, rec["expected"]) <= rec["tol_nt2ulp"], (rec, got)
