"""Folds of an expression in one pass (nt2g_eval_fold): the expression's value
at every element is computed inside the fold kernels, so sum(exp(x)*y),
sum(abs(x - y), 1), globalmax(exp(x) - y) read their input tables once and
write no temporary.

Parity:
  - equal, bit for bit, to nt2g_fold_f32 of the same expression first
    evaluated into an aligned table by the run-time compiled transform (same
    element policy and fold order): the fold kernels and their plan are the
    same, only the element source differs;
  - NT2 policy: bit-identical to the oracle's NT2 fold (index order, NT2's
    unfused float operations) of the oracle's NT2 evaluation of the elements;
  - fast policy: the FP64 result within 4 eps^2 sum|x| of the exact sum of the
    elements (the compensated fold's bound).
NT2's folds take the expression itself
(core/reduction/include/nt2/core/functions/scalar/inner_fold.hpp:23-49,
core/functions/details/fold_step.hpp:32-43, core/functions/simd/global.hpp:27-69)."""
import numpy as np
import pytest
import torch

from nt2_gb300 import expr as E

pytestmark = pytest.mark.gpu

EPS32 = float(np.finfo(np.float32).eps)


def _t(dev, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _materialized(lib, e_fn, tabs, elem_prec):
    """e evaluated into a fresh aligned table by the compiled transform."""
    out = torch.empty(tabs[0].numel(), device=tabs[0].device)
    E.assign([out], [e_fn(*[E.Table(t) for t in tabs])], precision=elem_prec, force_generic=1)
    return out


def _bits(t):
    return t.cpu().numpy().view(np.uint32) if t.dtype == torch.float32 else t.cpu().numpy()


PRECS = [("fast", 0, 0, 0), ("nt2", 1, 1, 1), ("nt2_elements", 2, 1, 0)]  # (name, fold prec, elements, order)


@pytest.mark.parametrize("name,prec,elem,order", PRECS, ids=[p[0] for p in PRECS])
@pytest.mark.parametrize("shape", [(1, 1 << 20, 1), (1, 4096, 256), (300, 2000, 3), (64, 512, 8), (1, 37, 3000),
                                   (5, 7, 1)],
                         ids=["global", "columns", "strided", "strided4", "short", "tiny"])
@pytest.mark.parametrize("op", ["sum", "max", "var", "nbtrue", "asum2"])
def test_fused_fold_equals_fold_of_materialized(lib, dev, name, prec, elem, order, shape, op):
    lo, inner, hi = shape
    n = lo * inner * hi
    rng = np.random.default_rng(7 + n)
    x, y = _t(dev, rng.standard_normal(n, dtype=np.float32)), _t(dev, rng.standard_normal(n, dtype=np.float32))
    fns = {"sum": lambda a, b: E.exp(a) * b, "max": lambda a, b: E.exp(a) - b, "var": lambda a, b: a * b + 1.0,
           "nbtrue": lambda a, b: a > b, "asum2": lambda a, b: E.abs_(a - b)}
    fn = fns[op]
    idx = op == "max"
    got = E.fold(fn(E.Table(x), E.Table(y)), op, shape, precision=prec, index=idx)
    m = _materialized(lib, fn, [x, y], elem)
    ref = lib.fold(m, lo, inner, hi, op, precision=order, index=idx)
    torch.cuda.synchronize()
    if idx:
        assert np.array_equal(_bits(got[0]), _bits(ref[0])) and np.array_equal(_bits(got[1]), _bits(ref[1]))
    else:
        assert np.array_equal(_bits(got), _bits(ref))


def test_nt2_policy_matches_the_oracle(lib, dev, oracle):
    """NT2's elements folded in NT2's order: sum(exp(x)*y) over 2^16 elements
    and sum(abs(x - y), 1) over a 256 x 300 table, bit-identical to the
    oracle's NT2 evaluation and fold."""
    rng = np.random.default_rng(11)
    n = 1 << 16
    x, y = rng.standard_normal(n, dtype=np.float32), rng.standard_normal(n, dtype=np.float32)
    got = E.fold(E.exp(E.Table(_t(dev, x))) * E.Table(_t(dev, y)), "sum", precision=lib.PREC_NT2)
    elems = (oracle.map_f32("exp", x) * y).astype(np.float32)
    ref = oracle.fold_nt2(elems, 1, n, 1, "sum")[0]
    assert np.array_equal(got.cpu().numpy().view(np.uint32), np.asarray(ref, np.float32).view(np.uint32))
    m, k = 256, 300
    a, b = rng.standard_normal(m * k, dtype=np.float32), rng.standard_normal(m * k, dtype=np.float32)
    got = E.fold(E.abs_(E.Table(_t(dev, a)) - E.Table(_t(dev, b))), "sum", (1, m, k), precision=lib.PREC_NT2)
    ref = oracle.fold_nt2(np.abs(a - b).astype(np.float32), 1, m, k, "sum")[0]
    assert np.array_equal(got.cpu().numpy().view(np.uint32), np.asarray(ref, np.float32).view(np.uint32))
    got = E.fold(E.abs_(E.Table(_t(dev, a)) - E.Table(_t(dev, b))), "max", (m, k, 1), precision=lib.PREC_NT2)
    ref = oracle.fold_nt2(np.abs(a - b).astype(np.float32), m, k, 1, "max")[0]
    assert np.array_equal(got.cpu().numpy().view(np.uint32), np.asarray(ref, np.float32).view(np.uint32))


@pytest.mark.parametrize("n", [1 << 24, (1 << 22) + 3])
def test_fast_sum_against_the_exact_sum(lib, dev, oracle, n):
    """sum(exp(x)*y) in one pass: the FP64 result within the compensated
    fold's bound of the exact sum of the same float elements; dot(x*2, y+1)
    likewise; misaligned views (one element in) give the same elements."""
    rng = np.random.default_rng(12)
    x, y = _t(dev, rng.standard_normal(n + 1, dtype=np.float32)), _t(dev, rng.standard_normal(n + 1, dtype=np.float32))
    for xs, ys in ((x[:n], y[:n]), (x[1:], y[1:])):
        for fn in (lambda a, b: E.exp(a) * b, lambda a, b: (a * 2.0) * (b + 1.0)):
            out, o64 = E.fold(fn(E.Table(xs), E.Table(ys)), "sum", out64=True)
            elems = _materialized(lib, fn, [xs, ys], 0).cpu().numpy()
            exact, absum = oracle.exact_sum(elems)
            err = abs(float(o64.item()) - exact)
            assert err <= 4 * EPS32 ** 2 * absum + 1e-15 * abs(exact), (err, exact, absum)
            assert float(out.item()) == np.float32(float(o64.item()))


def test_generative_and_uint8_folds(lib, dev, oracle):
    """A generative leaf folds without memory: sum(sinpi(linspace(0, 2, n)) * x);
    uint8 tables fold through a comparison: nbtrue(frame > bkg)."""
    n = 1 << 20
    rng = np.random.default_rng(13)
    x = _t(dev, rng.standard_normal(n, dtype=np.float32))
    e = E.sinpi(E.linspace(0, 2, n)) * E.Table(x)
    got = E.fold(e, "sum")
    out = torch.empty(n, device=dev)
    E.assign([out], [E.sinpi(E.linspace(0, 2, n)) * E.Table(x)], force_generic=1)
    assert np.array_equal(got.cpu().numpy().view(np.uint32), lib.fold(out, 1, n, 1, "sum").cpu().numpy().view(np.uint32))
    fr = _t(dev, rng.integers(0, 256, n, dtype=np.uint8))
    bkg = _t(dev, rng.integers(0, 256, n, dtype=np.uint8))
    for prec in (lib.PREC_FAST, lib.PREC_NT2):
        cnt = E.fold(E.Table(fr) > E.Table(bkg), "nbtrue", precision=prec)
        assert float(cnt.item()) == float(np.count_nonzero(fr.cpu().numpy() > bkg.cpu().numpy()))


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
def test_meanad_and_wmean(lib, dev, oracle, prec):
    """meanad of an expression (its two passes -- the mean, then |e - mean| --
    both over the expression's elements, no temporary) and NT2's wmean(a, w,
    dim) = rec(globalsum(w)) * sum(a .* w, dim): under the NT2 policy
    bit-identical to the oracle's NT2 folds of the same float elements; under
    the fast one within 2 ulp of the exact value."""
    rng = np.random.default_rng(31)
    m, k = 300, 1000
    a = (50.0 + rng.standard_normal(m * k)).astype(np.float32)
    b = rng.uniform(0.5, 2.0, m * k).astype(np.float32)
    ta, tb = _t(dev, a), _t(dev, b)
    elems = (a * b).astype(np.float32)  # a .* b rounded, as both policies compute it
    for shape in ((1, m, k), (m, k, 1)):
        got = E.fold(E.Table(ta) * E.Table(tb), "meanad", shape, precision=prec).cpu().numpy()
        if prec == 1:
            ref, _ = oracle.fold_nt2(elems, *shape, "meanad")
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), shape
        else:
            ref, _, _ = oracle.fold_ref(elems, *shape, "meanad")
            assert (np.abs(got - ref) <= 2 * np.spacing(np.abs(ref).astype(np.float32))).all(), shape
        wm = E.wmean(ta, tb, shape, precision=prec).cpu().numpy()
        if prec == 1:
            f = np.float32(1.0) / oracle.fold_nt2(b, 1, m * k, 1, "sum")[0][0]
            want = (f * oracle.fold_nt2(elems, *shape, "sum")[0]).astype(np.float32)
            assert np.array_equal(wm.view(np.uint32), want.view(np.uint32)), shape
        else:
            s, _, _ = oracle.fold_ref(elems, *shape, "sum")
            ref = s / oracle.fold_ref(b, 1, m * k, 1, "sum")[0][0]
            assert (np.abs(wm - ref) <= 2 * np.spacing(np.abs(ref).astype(np.float32))).all(), shape


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
def test_asump_and_normp(lib, dev, oracle, prec):
    """NT2's asump(a, p, dim) = sum(pow_abs(a, p), dim) and normp = pow(asump,
    rec(p)), pow(abs(a), p) folded in one pass: under the NT2 policy
    bit-identical to the oracle's NT2 pow and in-order fold; under the fast one
    asump within 5 ulp of FP64 (each term within 4, all positive: no
    cancellation) and normp within 4 + 5/p."""
    rng = np.random.default_rng(41)
    m, k = 300, 1000
    a = (rng.standard_normal(m * k) * np.exp2(rng.integers(-4, 4, m * k))).astype(np.float32)
    ta = _t(dev, a)
    a64 = np.abs(a.astype(np.float64))
    for p in (3.0, 1.5, 0.5):
        elems = oracle.pow_f32(np.abs(a), np.full_like(a, np.float32(p)))
        inv = np.float32(1.0) / np.float32(p)
        for shape in ((1, m, k), (m, k, 1)):
            got_s = E.asump(ta, p, shape, precision=prec).cpu().numpy()
            got_n = E.normp(ta, p, shape, precision=prec).cpu().numpy()
            if prec == 1:
                ref, _ = oracle.fold_nt2(elems, *shape, "sum")
                assert np.array_equal(got_s.view(np.uint32), ref.view(np.uint32)), (p, shape)
                want = oracle.pow_f32(ref, np.full_like(ref, inv))
                assert np.array_equal(got_n.view(np.uint32), want.view(np.uint32)), (p, shape)
            else:
                lo, inner, hi = shape
                s64 = (a64 ** p).reshape(hi, inner, lo).sum(axis=1).ravel()
                assert (np.abs(got_s - s64) <= 5 * np.spacing(s64.astype(np.float32))).all(), (p, shape)
                # the sum's 5 ulp scaled by 1/p through the root, plus the root's own 4
                n64 = s64 ** (1.0 / p)
                tol = 4 + 5 / p
                assert (np.abs(got_n - n64) <= tol * np.spacing(n64.astype(np.float32))).all(), (p, shape)


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
def test_nanasum2(lib, dev, oracle, prec):
    """NT2's nanasum2(a, dim) = sum(if_zero_else(is_nan(a), sqr_abs(a)), dim),
    the select and the square folded in one pass: NaNs contribute nothing;
    NT2 policy bit-identical to the oracle's in-order fold, fast within 1 ulp."""
    rng = np.random.default_rng(43)
    m, k = 300, 1000
    a = rng.standard_normal(m * k).astype(np.float32)
    a[rng.integers(0, a.size, 5000)] = np.nan
    sq = np.where(np.isnan(a), np.float32(0), (a * a).astype(np.float32)).astype(np.float32)
    for shape in ((1, m, k), (m, k, 1), (1, m * k, 1)):
        got = E.nanasum2(_t(dev, a), shape, precision=prec).cpu().numpy()
        if prec == 1:
            ref, _ = oracle.fold_nt2(sq, *shape, "sum")
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), shape
        else:
            ref, _, _ = oracle.fold_ref(sq, *shape, "sum")
            assert (np.abs(got - ref) <= np.spacing(np.abs(ref).astype(np.float32))).all(), shape
