"""Reductions along one dimension (sum(a, dim), max(a, [], dim), mean, norm2,
...) of tables viewed as [lo, inner, hi], against the oracle.

NT2 policy: bit-identical to the oracle's restatement of NT2's in-order
per-output fold (values and max/min positions).  Fast policy: sum-type results
within one float ulp of the exact value (compensated FP32 chunks combined in
FP64), products within two ulps, max/min and positions identical to NT2's
order on NaN-free data, a NaN propagated with its first position.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SHAPES = [
    (1, 4096, 4096),      # dim 1 of a 4096 x 4096 table: one chunk per column
    (4096, 4096, 1),      # dim 2 of the same table: strided, 4 outputs per thread
    (1, 1 << 22, 1),      # global: many chunks, two-pass combine
    (1, 17, 10000),       # short columns: one thread per column
    (1, 100003, 7),       # ragged, unaligned columns
    (1001, 33, 77),       # middle dimension of a 3-D table, lo not a multiple of 4
    (64, 1 << 16, 1),     # few long rows: chunked strided fold
    (3, 5, 2),
    (1, 0, 5),            # empty fold: neutral element
]
OPS = ["sum", "prod", "max", "min", "mean", "asum1", "asum2", "norm2"]


def _data(shape, op, seed):
    lo, inner, hi = shape
    rng = np.random.default_rng(seed)
    n = lo * inner * hi
    if op == "prod":  # keep products finite: factors near 1
        x = rng.uniform(0.999, 1.001, n)
    else:
        x = rng.standard_normal(n) * np.exp2(rng.integers(-8, 8, n))
    x = x.astype(np.float32)
    if op in ("max", "min") and n > 10:  # ties, signed zeros
        x[rng.integers(0, n, n // 50)] = 0.0
        x[rng.integers(0, n, n // 50)] = -0.0
        x[rng.integers(0, n, n // 100)] = x.max() if op == "max" else x.min()
    return x


def _same_bits(a, b):
    """Bitwise equality, any NaN equal to any NaN (NaN payloads differ by platform)."""
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    return bool(np.all((a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))))


def _ulp32(v):
    return np.spacing(np.abs(v).astype(np.float32)).astype(np.float64)


@pytest.mark.parametrize("shape", SHAPES, ids=[f"{a}x{b}x{c}" for a, b, c in SHAPES])
@pytest.mark.parametrize("op", OPS)
def test_fold_nt2_policy_bit_exact(lib, dev, oracle, shape, op):
    lo, inner, hi = shape
    x = _data(shape, op, 11)
    tx = torch.from_numpy(x).to(dev)
    want_idx = op in ("max", "min")
    got = lib.fold(tx, lo, inner, hi, op, precision=lib.PREC_NT2, index=want_idx)
    torch.cuda.synchronize()
    ref, ridx = oracle.fold_nt2(x, lo, inner, hi, op)
    out = (got[0] if want_idx else got).cpu().numpy()
    assert _same_bits(out, ref)
    if want_idx:
        assert np.array_equal(got[1].cpu().numpy(), ridx)


@pytest.mark.parametrize("shape", SHAPES, ids=[f"{a}x{b}x{c}" for a, b, c in SHAPES])
@pytest.mark.parametrize("op", OPS)
def test_fold_fast_policy(lib, dev, oracle, shape, op):
    lo, inner, hi = shape
    x = _data(shape, op, 12)
    tx = torch.from_numpy(x).to(dev)
    want_idx = op in ("max", "min")
    got = lib.fold(tx, lo, inner, hi, op, index=want_idx)
    torch.cuda.synchronize()
    ref, asum, ridx = oracle.fold_ref(x, lo, inner, hi, op)
    out = (got[0] if want_idx else got).cpu().numpy()
    if inner == 0:
        nt2, _ = oracle.fold_nt2(x, lo, inner, hi, op)
        assert _same_bits(out, nt2)
        return
    if want_idx:
        assert np.array_equal(out.view(np.uint32), ref.astype(np.float32).view(np.uint32))
        assert np.array_equal(got[1].cpu().numpy(), ridx)
        nt2, nidx = oracle.fold_nt2(x, lo, inner, hi, op)  # no NaN here: equal to NT2's order
        assert np.array_equal(out.view(np.uint32), nt2.view(np.uint32)) and np.array_equal(got[1].cpu().numpy(), nidx)
        return
    err = np.abs(out.astype(np.float64) - ref)
    tol = (2.0 if op == "prod" else 1.0) * _ulp32(ref)
    assert (err <= tol).all(), (op, shape, float((err / _ulp32(ref)).max()))


def test_fold_max_min_nan_propagates(lib, dev, oracle):
    x = np.random.default_rng(13).standard_normal(3 * 1000 * 5).astype(np.float32)
    x[[7, 2500, 9000, 9001]] = np.nan
    tx = torch.from_numpy(x).to(dev)
    for lo, inner, hi in ((1, 3000, 5), (3, 1000, 5)):
        for op in ("max", "min"):
            out, idx = lib.fold(tx, lo, inner, hi, op, index=True)
            ref, _, ridx = oracle.fold_ref(x, lo, inner, hi, op)
            torch.cuda.synchronize()
            o = out.cpu().numpy()
            assert np.array_equal(np.isnan(o), np.isnan(ref)) and np.array_equal(o[~np.isnan(o)],
                                                                                 ref[~np.isnan(ref)].astype(np.float32))
            assert np.array_equal(idx.cpu().numpy(), ridx)


def test_fold_global_matches_reduce_entry(lib, dev):
    """globalsum through the fold family agrees with the dedicated sum kernel
    to within one float ulp of the exact value (both compensated)."""
    n = (1 << 24) + 3
    x = np.random.default_rng(14).standard_normal(n).astype(np.float32)
    tx = torch.from_numpy(x).to(dev)
    a = lib.fold(tx, 1, n, 1, "sum").item()
    b = lib.Reducer(dev)(tx)[1].item()
    assert abs(a - b) <= np.spacing(np.float32(abs(b)))


VAR_OPS = ["var", "stdev", "var1", "stdev1", "meanad"]  # the folds of deviations from each output's mean


def _offset_data(shape, seed):
    lo, inner, hi = shape
    rng = np.random.default_rng(seed)
    # an offset far from zero exercises the centring; spreads vary per element
    return (1000.0 + rng.standard_normal(lo * inner * hi) * np.exp2(rng.integers(-4, 4, lo * inner * hi))).astype(np.float32)


@pytest.mark.parametrize("shape", [s for s in SHAPES if s[0] * s[1] * s[2] <= (1 << 20)],
                         ids=lambda s: f"{s[0]}x{s[1]}x{s[2]}")
@pytest.mark.parametrize("op", VAR_OPS)
def test_fold_var_nt2_policy_bit_exact(lib, dev, oracle, shape, op):
    """var/stdev under NT2's policy: NT2's float mean, the in-order sum of
    squared deviations, f = rec(n - 1) (or rec(n)), bit-identical; meanad:
    rec(n) times the in-order sum of |x - mean| (mean(abs(center(a))))."""
    lo, inner, hi = shape
    x = _offset_data(shape, 21)
    got = lib.fold(torch.from_numpy(x).to(dev), lo, inner, hi, op, precision=lib.PREC_NT2)
    torch.cuda.synchronize()
    ref, _ = oracle.fold_nt2(x, lo, inner, hi, op)
    assert _same_bits(got.cpu().numpy(), ref)


@pytest.mark.parametrize("shape", SHAPES, ids=[f"{a}x{b}x{c}" for a, b, c in SHAPES])
@pytest.mark.parametrize("op", VAR_OPS)
def test_fold_var_fast_policy(lib, dev, oracle, shape, op):
    """var/stdev/meanad under the fast policy: within 2 float ulps of the
    exact value (FP64 reference about the exact mean), offset data included
    (meanad carries the mean's rounding error into every deviation)."""
    lo, inner, hi = shape
    x = _offset_data(shape, 22)
    got = lib.fold(torch.from_numpy(x).to(dev), lo, inner, hi, op).cpu().numpy()
    torch.cuda.synchronize()
    ref, _, _ = oracle.fold_ref(x, lo, inner, hi, op)
    if inner == 0:
        nt2, _ = oracle.fold_nt2(x, lo, inner, hi, op)
        assert _same_bits(got, nt2)
        return
    err = np.abs(got.astype(np.float64) - ref)
    tol = 2.0 * _ulp32(ref) + 1e-30
    assert (err <= tol).all(), (op, shape, float((err / _ulp32(ref)).max()))


COUNT_OPS = ["nbtrue", "all", "any", "none", "nansum", "nanmean"]


def _zeros_nans(shape, seed, zeros=True):
    lo, inner, hi = shape
    n = lo * inner * hi
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal(n) * np.exp2(rng.integers(-6, 6, n))).astype(np.float32)
    if n > 10:
        if zeros:
            x[rng.integers(0, n, n // 3)] = 0.0
            x[rng.integers(0, n, n // 50)] = -0.0
        x[rng.integers(0, n, n // 40)] = np.nan
    return x


@pytest.mark.parametrize("shape", [s for s in SHAPES if s[0] * s[1] * s[2] <= (1 << 20)],
                         ids=lambda s: f"{s[0]}x{s[1]}x{s[2]}")
@pytest.mark.parametrize("op", COUNT_OPS)
def test_fold_counts_nan_nt2_policy_bit_exact(lib, dev, oracle, shape, op):
    lo, inner, hi = shape
    x = _zeros_nans(shape, 31)
    got = lib.fold(torch.from_numpy(x).to(dev), lo, inner, hi, op, precision=lib.PREC_NT2)
    torch.cuda.synchronize()
    ref, _ = oracle.fold_nt2(x, lo, inner, hi, op)
    assert _same_bits(got.cpu().numpy(), ref)


@pytest.mark.parametrize("shape", SHAPES, ids=[f"{a}x{b}x{c}" for a, b, c in SHAPES])
@pytest.mark.parametrize("op", COUNT_OPS)
def test_fold_counts_nan_fast_policy(lib, dev, oracle, shape, op):
    """Counts and the logical folds exact; nansum within one ulp of the exact
    sum of the non-NaN elements, nanmean within two."""
    lo, inner, hi = shape
    x = _zeros_nans(shape, 32)
    got = lib.fold(torch.from_numpy(x).to(dev), lo, inner, hi, op).cpu().numpy()
    torch.cuda.synchronize()
    ref, _, _ = oracle.fold_ref(x, lo, inner, hi, op)
    if op in ("nbtrue", "all", "any", "none"):
        assert np.array_equal(got, ref.astype(np.float32))
        return
    err = np.abs(got.astype(np.float64) - ref)
    tol = (2.0 if op == "nanmean" else 1.0) * _ulp32(ref) + 1e-37
    assert (err <= tol).all(), (op, shape, float((err / _ulp32(ref)).max()))


def test_fold_all_any_none_edges(lib, dev):
    """all of nonzero data is 1, any/none of zeros are 0/1, NaN counts as true,
    and the empty fold gives all = 1, any = 0, none = 1."""
    z = torch.zeros(3 * 4096, device=dev)
    o = torch.ones(3 * 4096, device=dev)
    nan = torch.full((3 * 4096,), float("nan"), device=dev)
    for prec in (lib.PREC_FAST, lib.PREC_NT2):
        f = lambda t, op: lib.fold(t, 3, 4096, 1, op, precision=prec).cpu().numpy()  # noqa: E731
        assert (f(o, "all") == 1).all() and (f(z, "all") == 0).all() and (f(nan, "all") == 1).all()
        assert (f(z, "any") == 0).all() and (f(o, "any") == 1).all() and (f(z, "none") == 1).all()
        assert (f(nan, "nbtrue") == 4096).all() and (f(nan, "nansum") == 0).all() and (f(nan, "nanmean") == 0).all()
        e = torch.zeros(0, device=dev)
        g = lambda op: lib.fold(e, 1, 0, 5, op, precision=prec).cpu().numpy()  # noqa: E731
        assert (g("all") == 1).all() and (g("any") == 0).all() and (g("none") == 1).all() and (g("nbtrue") == 0).all()
