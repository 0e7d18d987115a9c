"""median / medianad along a dimension and globalmedian / globalmedianad
(NT2's core/reduction/include/nt2/core/functions/expr/median.hpp and
expr/medianad.hpp) on the GPU against the oracle's restatement (sort each
slice, take the middle element or meanof of the two middle ones): equal
results on every shape, in shared memory (slices up to 40960 elements) and in
the global passes beyond; ties, signed zeros, infinities, NaN slices, empty
slices, strided slices (dim > 1); NT2's own known answers (median.cpp,
medianad.cpp); a 2^26-element global median against numpy's partition."""
import json
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "nt2_unit_vectors.json")))


def _eq(a, b):
    """Equal as floats (-0 == +0: NT2's sort orders the two zeros either way), NaN where NaN."""
    return np.array_equal(np.isnan(a), np.isnan(b)) and bool((a[~np.isnan(a)] == b[~np.isnan(b)]).all())


def _data(rng, n, kind):
    if kind == "normal":
        return rng.standard_normal(n).astype(np.float32)
    if kind == "ties":  # few distinct values: many equal keys at the middle
        return rng.integers(-3, 4, n).astype(np.float32)
    if kind == "zeros":  # signed zeros around the middle, a few infinities
        x = rng.choice(np.float32([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf]), n, p=[.35, .35, .1, .1, .05, .05])
        return x.astype(np.float32)
    return (rng.standard_normal(n) * np.exp2(rng.integers(-60, 60, n))).astype(np.float32)  # wide exponents


@pytest.mark.parametrize("shape", [(1, 1, 5), (1, 2, 7), (1, 3, 9), (1, 4, 6), (1, 7, 33), (1, 8, 33), (1, 31, 17),
                                   (1, 32, 17), (1, 33, 17), (1, 256, 9), (1, 1000, 5), (1, 1001, 5),
                                   (1, 4096, 3), (1, 40960, 2), (1, 40961, 2), (1, 100000, 3), (1, 131072, 2),
                                   (3, 10, 4), (1000, 77, 1), (4096, 50, 2), (7, 9, 11), (4, 50000, 1),
                                   (3, 45000, 2)],
                         ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("kind", ["normal", "ties", "zeros", "wide"])
def test_median_against_oracle(lib, dev, oracle, shape, kind):
    lo, inner, hi = shape
    rng = np.random.default_rng(lo * 7919 + inner * 31 + hi)
    x = _data(rng, lo * inner * hi, kind)
    tx = torch.from_numpy(x).to(dev)
    for op in ("median", "medianad"):
        got = lib.median(tx, lo, inner, hi, op).cpu().numpy()
        ref = oracle.median(x, lo, inner, hi, ad=op == "medianad")
        assert _eq(got, ref), (op, np.flatnonzero(~((got == ref) | (np.isnan(got) & np.isnan(ref))))[:5])


def test_median_nan_and_empty_slices(lib, dev, oracle):
    """A slice holding a NaN gives NaN, its neighbours their medians; an empty
    dimension gives NaN; no slices, no work."""
    x = np.arange(60, dtype=np.float32)
    x[[7, 33]] = np.nan
    tx = torch.from_numpy(x).to(dev)
    for shape in ((1, 10, 6), (6, 10, 1), (1, 60, 1)):
        for op in ("median", "medianad"):
            got = lib.median(tx, *shape, op).cpu().numpy()
            assert _eq(got, oracle.median(x, *shape, ad=op == "medianad")), (shape, op)
    big = np.random.default_rng(3).standard_normal(3 * 50000).astype(np.float32)
    big[50000 + 12345] = np.nan  # the second of three long slices (global passes)
    got = lib.median(torch.from_numpy(big).to(dev), 1, 50000, 3).cpu().numpy()
    assert np.isnan(got[1]) and not np.isnan(got[0]) and not np.isnan(got[2])
    assert _eq(got, oracle.median(big, 1, 50000, 3))
    empty = lib.median(torch.zeros(1, device=dev), 5, 0, 1).cpu().numpy()
    assert empty.shape == (5,) and np.isnan(empty).all()
    assert lib.median(torch.zeros(1, device=dev), 0, 5, 3).numel() == 0


@pytest.mark.parametrize("rec", [r for r in GOLDEN if r["fn"] in ("median", "medianad")],
                         ids=lambda r: f"{r['fn']}{tuple(r['shape'])}")
def test_median_nt2_unit_tests(lib, dev, rec):
    got = lib.median(torch.tensor(rec["x"], dtype=torch.float32, device=dev), *rec["shape"], rec["fn"]).cpu().numpy()
    assert np.array_equal(got, np.float32(rec["expected"])), (got, rec)


def test_global_median_large(lib, dev):
    """globalmedian of 2^26 + 1 and 2^26 elements (global passes) equals the
    middle order statistic(s) numpy's partition finds."""
    rng = np.random.default_rng(8)
    for n in ((1 << 26) + 1, 1 << 26):
        x = (rng.standard_normal(n) * 10).astype(np.float32)
        got = float(lib.median(torch.from_numpy(x).to(dev), 1, n, 1).cpu().numpy()[0])
        mid = n >> 1
        if n & 1:
            want = np.partition(x, mid)[mid]
        else:
            p = np.partition(x, [mid - 1, mid])
            a, b = p[mid - 1], p[mid]
            want = np.float32(a + np.float32(np.float32(b - a) * np.float32(0.5)))
        assert got == want, (n, got, want)



@pytest.mark.parametrize("prec", [1, 0], ids=["nt2", "fast"])
def test_trapz(lib, dev, oracle, prec):
    """trapz (unit spacing) along every kind of dimension: under the NT2 policy
    bit-identical to the oracle's NT2 order (neighbour sums folded in index
    order, halved); under the fast one within 1 ulp of the FP64 value plus the
    float rounding of the sum's magnitude; slices of 0 and 1 elements give 0;
    NT2's known answers (trapz.cpp)."""
    rng = np.random.default_rng(71)
    for shape in ((1, 1000, 300), (300, 1000, 1), (7, 33, 5), (1, 1 << 20, 1), (4, 1, 3), (3, 0, 2), (1, 2, 5)):
        lo, inner, hi = shape
        x = rng.standard_normal(max(lo * inner * hi, 1)).astype(np.float32)
        got = lib.trapz(torch.from_numpy(x).to(dev), lo, inner, hi, precision=prec).cpu().numpy()
        if prec == 1:
            assert np.array_equal(got.view(np.uint32), oracle.trapz_nt2(x, lo, inner, hi).view(np.uint32)), shape
        else:
            v = x[:lo * inner * hi].astype(np.float64).reshape(hi, inner, lo)
            ref = (0.5 * (v[:, 1:, :] + v[:, :-1, :]).sum(axis=1)).ravel() if inner > 1 else np.zeros(lo * hi)
            mag = (np.abs(v).sum(axis=1)).ravel()
            assert (np.abs(got - ref) <= np.spacing(np.abs(ref).astype(np.float32)) + 2e-7 * mag).all(), shape
    for rec in [r for r in GOLDEN if r["fn"] == "trapz"]:
        got = lib.trapz(torch.tensor(rec["x"], dtype=torch.float32, device=dev), *rec["shape"], precision=prec)
        assert np.array_equal(got.cpu().numpy(), np.float32(rec["expected"])), rec
