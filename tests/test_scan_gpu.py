"""Cumulative functions along one dimension (cumsum, cumprod, cummax, cummin)
of tables viewed as [lo, inner, hi], against the oracle.

NT2 policy: bit-identical to the oracle's restatement of NT2's in-order scan.
Fast policy: cumsum within an ulp of the exact prefix (plus 1e-12 of the
running sum of |x|, the compensated FP32/FP64 error), cumprod within two
ulps of the long-double product, cummax/cummin bit-identical to NT2's order,
NaNs and signed zeros included.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SHAPES = [
    (1, 4096, 4096),      # dim 1 of a 4096 x 4096 table: one chunk per column
    (4096, 4096, 1),      # dim 2: strided, 4 segments per thread
    (1, 1 << 22, 1),      # one long segment: three-phase
    (1, 17, 10000),       # short columns
    (1, 100003, 7),       # ragged, unaligned columns
    (1001, 33, 77),       # middle dimension of a 3-D table
    (64, 1 << 16, 1),     # few long strided segments: chunked
    (3, 5, 2),
]
OPS = ["sum", "prod", "max", "min"]


def _data(shape, op, seed, nan=False):
    lo, inner, hi = shape
    n = lo * inner * hi
    rng = np.random.default_rng(seed)
    if op == "prod":
        x = rng.uniform(0.999, 1.001, n)
    else:
        x = rng.standard_normal(n) * np.exp2(rng.integers(-8, 8, n))
    x = x.astype(np.float32)
    if op in ("max", "min") and n > 10:
        x[rng.integers(0, n, n // 50)] = 0.0
        x[rng.integers(0, n, n // 50)] = -0.0
        if nan:
            x[rng.integers(0, n, n // 100 + 1)] = np.nan
    return x


def _same_bits(a, b):
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    return bool(np.all((a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))))


@pytest.mark.parametrize("shape", SHAPES, ids=[f"{a}x{b}x{c}" for a, b, c in SHAPES])
@pytest.mark.parametrize("op", OPS)
def test_scan_nt2_policy_bit_exact(lib, dev, oracle, shape, op):
    x = _data(shape, op, 31, nan=True)
    got = lib.scan(torch.from_numpy(x).to(dev), *shape, op, precision=lib.PREC_NT2)
    torch.cuda.synchronize()
    assert _same_bits(got.cpu().numpy(), oracle.scan_nt2(x, *shape, op))


@pytest.mark.parametrize("shape", SHAPES, ids=[f"{a}x{b}x{c}" for a, b, c in SHAPES])
@pytest.mark.parametrize("op", OPS)
def test_scan_fast_policy(lib, dev, oracle, shape, op):
    x = _data(shape, op, 32, nan=True)
    got = lib.scan(torch.from_numpy(x).to(dev), *shape, op).cpu().numpy()
    torch.cuda.synchronize()
    if op in ("max", "min"):
        assert _same_bits(got, oracle.scan_nt2(x, *shape, op))
        return
    if op == "sum":
        ref, absrun = oracle.cumsum_exact(x, *shape)
        tol = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64) + 1e-12 * absrun
    else:
        x64 = x.astype(np.float64).reshape(shape[2], shape[1], shape[0])  # [hi][inner][lo] in C order
        ref = np.cumprod(x64, axis=1).ravel()
        tol = 2 * np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    err = np.abs(got.astype(np.float64) - ref)
    assert (err <= tol).all(), (op, shape, float((err / np.maximum(tol, 1e-300)).max()))


def test_scan_in_place(lib, dev, oracle):
    shape = (1, 100000, 3)
    x = _data(shape, "sum", 33)
    t = torch.from_numpy(x).to(dev)
    lib.scan(t, *shape, "max", out=t)
    torch.cuda.synchronize()
    assert _same_bits(t.cpu().numpy(), oracle.scan_nt2(x, *shape, "max"))
