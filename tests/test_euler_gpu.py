"""erf, erfcx, gamma, gammaln and the exponential extras (expx2, exprecneg,
exprecnegc, sqrt1pm1; logspace_add, logspace_sub and the real* aliases as
NT2's compositions) on the GPU.

NT2 policy: bit-identical to the oracle's restatement of NT2's float
algorithms.  Fast policy: against FP64 within the tolerances below, with
NT2's NaN positions.  Where NT2's float algorithm loses accuracy the fast
policy computes the function another way: erf above 2/3 and erfcx from the fast
erfc tail, e^(x^2) and e^(-1/x) with the argument split exactly, sqrt1pm1
without the cancelling branch, gamma with its product carried in float-float,
erfcinv with erfinv's second polynomial up to w = 16 and one Newton step on
erfcx beyond it.
gammaln follows NT2's algorithm in both policies; around Gamma's minimum
(x = 1.46) its x B(x) - log(x) form cancels to 6.3 ulp, and on the negative
axis its reflection cancels near the zeros and poles (an absolute error of a
few ulp of the terms there).
NT2's gamma steps x down one unit at a time; its product is +inf long before
64 and the steps never end from 2^24 on, so both policies return +inf from 64.
NT2's exp overflows from Maxlog (88.376) on, below log(FLT_MAX); results past
e^Maxlog are +inf in both policies and are not compared with FP64.  NT2's
expx2 is NaN from about 1.7e38 on (its 2m overflows while f is 0), and so is
erfcx below -1.7e38; the fast policy returns +inf there.
"""
import json
import os

import numpy as np
import pytest
import torch

from helpers import nt2_ulpdist, std_ulp

pytestmark = pytest.mark.gpu

DEVICE = ["erf", "erfcx", "expx2", "gamma", "gammaln", "exprecneg", "exprecnegc", "sqrt1pm1", "erfinv", "erfcinv"]
FAST_TOL = dict(erf=2.5, erfcx=3.0, expx2=2.0, gamma=3.5, gammaln=6.5, exprecneg=2.0, exprecnegc=2.5,
                sqrt1pm1=2.0, erfinv=3.5, erfcinv=4.0)


def domain(fn, n, seed):
    """Seeded inputs covering each function's bands and edges."""
    rng = np.random.default_rng(seed)
    if fn == "erf":
        parts = [rng.uniform(-1, 1, n), rng.uniform(-6, 6, n), np.exp(rng.uniform(np.log(1e-30), 0, n))]
    elif fn == "erfcx":
        parts = [rng.uniform(-2, 2, n), rng.uniform(-9.5, 30, n), np.exp(rng.uniform(0, np.log(1e30), n))]
    elif fn == "expx2":
        parts = [rng.uniform(-9.5, 9.5, n), rng.uniform(-1, 1, n)]
    elif fn == "gamma":
        parts = [rng.uniform(0, 36, n), rng.uniform(-42, 0, n), np.exp(rng.uniform(np.log(1e-30), 0, n)),
                 rng.integers(-40, 40, n).astype(np.float64)]
    elif fn == "gammaln":
        parts = [rng.uniform(0, 10, n), rng.uniform(-50, 0, n), np.exp(rng.uniform(np.log(1e-30), np.log(1e36), n))]
    elif fn == "erfinv":
        parts = [rng.uniform(-1, 1, n), 1 - np.exp(rng.uniform(np.log(1e-7), 0, n)), rng.uniform(-1.01, -0.99, n)]
    elif fn == "erfcinv":
        parts = [rng.uniform(0, 2, n), np.exp(rng.uniform(np.log(1e-38), 0, n)), 2 - np.exp(rng.uniform(np.log(1e-7), 0, n))]
    elif fn in ("exprecneg", "exprecnegc"):
        parts = [rng.uniform(-2, 2, n), np.exp(rng.uniform(np.log(1e-3), np.log(1e30), n)) * rng.choice([-1.0, 1.0], n)]
    else:  # sqrt1pm1
        parts = [rng.uniform(-1, 1, n), np.exp(rng.uniform(np.log(1e-30), np.log(1e30), n)), rng.uniform(-1, 3, n)]
    return np.concatenate(parts).astype(np.float32)


SPECIALS = np.float32([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, 0.5, -0.5, 2.0, -2.0, 0.6666666, 0.6666667,
                       3.0, 6.5, 1.5, 1.25, 0.75, 2.5, 9.4, 9.5, 16.0, 33.0, -33.0, -33.5, 35.0, 35.04, 36.0, 64.0,
                       65.0, 1e4, 1e-45, 1e-38, 1e30, 3.4e38, -3.4e38, 16777216.0, 33554432.0])


def _run(lib, dev, fn, x, prec):
    tx = torch.from_numpy(x).to(dev)
    ty = torch.empty_like(tx)
    lib.map_f32(fn, tx, ty, precision=prec)
    torch.cuda.synchronize()
    return ty.cpu().numpy()


def _same(a, b):
    return (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))


@pytest.mark.parametrize("fn", DEVICE)
def test_nt2_policy_bit_exact(lib, dev, oracle, fn):
    x = np.concatenate([domain(fn, 1 << 17, 11), SPECIALS, -SPECIALS])
    got = _run(lib, dev, fn, x, lib.PREC_NT2)
    ref = oracle.map_f32(fn, x)
    same = _same(got, ref)
    assert same.all(), f"{(~same).sum()} differ, first at x={x[~same][:5]} got {got[~same][:5]} want {ref[~same][:5]}"


@pytest.mark.parametrize("fn", DEVICE)
def test_fast_policy_accuracy(lib, dev, oracle, fn):
    x = np.concatenate([domain(fn, 1 << 17, 12), SPECIALS, -SPECIALS])
    got = _run(lib, dev, fn, x, lib.PREC_FAST)
    ref = oracle.map_f64(fn, x)
    nt2 = oracle.map_f32(fn, x)
    keep = ~(np.abs(x) > 1e38) if fn in ("expx2", "erfcx") else np.ones(x.shape, bool)
    nan_got, nan_nt2 = np.isnan(got[keep]), np.isnan(nt2[keep])
    assert np.array_equal(nan_got, nan_nt2), x[keep][nan_got != nan_nt2][:8]
    maxexp = np.exp(np.float64(np.uint32(0x42b0c0a5).view(np.float32)))
    m = np.isfinite(ref) & (np.abs(ref) >= np.finfo(np.float32).tiny) & (np.abs(ref) < maxexp) & ~np.isnan(nt2)
    m &= np.abs(ref) < maxexp * (1 - 1e-5)  # results at the threshold round either way
    dist = np.abs(x - np.round(np.where(np.isfinite(x), x, 0)))  # to the nearest integer
    if fn == "gamma":  # within 1e-3 of a pole the float argument itself decides the value
        m &= ~((x < 0) & (dist < 1e-3))
    if fn == "gammaln":
        # on the negative axis NT2's reflection -log|x sinpi(x)/pi| - gammaln(|x|) cancels near the zeros and
        # the poles: there the error is absolute, a few ulp of the terms (which grow like |x| log|x|)
        near = m & (x < 0) & ((np.abs(ref) <= 1.0) | (dist < 1e-3))
        scale = np.maximum(1.0, np.abs(x[near]) * np.log1p(np.abs(x[near])))
        assert (np.abs(got[near] - ref[near]) <= 5e-6 * scale).all()
        m &= ~near
    e = std_ulp(got[m], ref[m])
    print(f"\n{fn}: fast policy vs FP64 max {e.max():.3f} mean {e.mean():.4f} ulp over {m.sum()} points")
    assert e.max() <= FAST_TOL[fn], f"max {e.max()} ulp at x={x[m][np.argmax(e)]}"


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
def test_golden_values(lib, dev, prec):
    golden = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "nt2_unit_vectors.json")))
    recs = [r for r in golden if r["fn"] in DEVICE]
    assert len(recs) >= 55
    for fn in sorted({r["fn"] for r in recs}):
        rs = [r for r in recs if r["fn"] == fn]
        got = _run(lib, dev, fn, np.float32([r["x"] for r in rs]), prec)
        for g, r in zip(got, rs):
            assert nt2_ulpdist(g, r["expected"]) <= r["tol_nt2ulp"], (r, g)


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
def test_logspace_and_real_aliases(lib, dev, oracle, prec):
    from nt2_gb300 import expr as E
    rng = np.random.default_rng(13)
    a = np.concatenate([rng.uniform(-80, 80, 1 << 16), SPECIALS, SPECIALS]).astype(np.float32)
    b = np.concatenate([rng.uniform(-80, 80, 1 << 16), SPECIALS, SPECIALS[::-1]]).astype(np.float32)
    ta, tb = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
    outs = [torch.empty_like(ta) for _ in range(4)]
    A, B = E.Table(ta), E.Table(tb)
    E.assign(outs, [E.logspace_add(A, B), E.logspace_sub(A, B), E.realsqrt(E.abs_(A)), E.reallog(E.abs_(B))],
             precision=prec)
    got = [o.cpu().numpy() for o in outs]
    L = oracle.lib()
    want_add = np.float32([L.o_logspace_add(float(p), float(q)) for p, q in zip(a, b)])
    want_sub = np.float32([L.o_logspace_sub(float(p), float(q)) for p, q in zip(a, b)])
    if prec == 1:
        assert _same(got[0], want_add).all() and _same(got[1], want_sub).all()
        assert _same(got[2], oracle.map_f32("sqrt", np.abs(a))).all()
        assert _same(got[3], oracle.map_f32("log", np.abs(b))).all()
    else:
        with np.errstate(invalid="ignore"):
            ref = np.logaddexp(a.astype(np.float64), b.astype(np.float64))
        m = np.isfinite(ref) & (np.abs(ref) > 1e-30) & np.isfinite(a) & np.isfinite(b)
        assert std_ulp(got[0][m], ref[m]).max() <= 3.5
    golden = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "nt2_unit_vectors.json")))
    for name in ("logspace_add", "logspace_sub"):
        recs = [r for r in golden if r["fn"] == name]
        assert len(recs) >= 7
        ta = torch.tensor([r["x"] for r in recs], dtype=torch.float32, device=dev)
        tb = torch.tensor([r["y"] for r in recs], dtype=torch.float32, device=dev)
        ty = torch.empty_like(ta)
        E.assign([ty], [getattr(E, name)(E.Table(ta), E.Table(tb))], precision=prec)
        for g, r in zip(ty.cpu().numpy(), recs):
            assert nt2_ulpdist(g, r["expected"]) <= r["tol_nt2ulp"], (r, g)


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
def test_digamma_signgam_beta_betaln(lib, dev, oracle, prec):
    """digamma (NT2's double algorithm rounded to float, in both policies) and
    signgam: bit-identical to the oracle; beta and betaln as NT2 composes them
    (signgam, gammaln, exp): bit-identical to the oracle under the NT2 policy,
    within a few ulp of the cancelling gammaln terms of FP64 under the fast
    one; NT2's own known answers (digamma.cpp, signgam.cpp, beta.cpp,
    betaln.cpp) in both."""
    from nt2_gb300 import expr as E
    rng = np.random.default_rng(21)
    x = np.concatenate([rng.uniform(-30, 40, 1 << 17), np.exp(rng.uniform(-20, 30, 1 << 15)), SPECIALS,
                        -SPECIALS, np.arange(-8, 9, dtype=np.float64)]).astype(np.float32)
    for fn in ("digamma", "signgam"):
        got = _run(lib, dev, fn, x, prec)
        ref = oracle.map_f32(fn, x)
        same = _same(got, ref)
        assert same.all(), (fn, x[~same][:5], got[~same][:5], ref[~same][:5])
    golden = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "nt2_unit_vectors.json")))
    for fn in ("digamma", "signgam"):
        rs = [r for r in golden if r["fn"] == fn]
        assert len(rs) >= 4
        got = _run(lib, dev, fn, np.float32([r["x"] for r in rs]), prec)
        for g, r in zip(got, rs):
            assert nt2_ulpdist(g, r["expected"]) <= r["tol_nt2ulp"], (r, g)
    a = np.concatenate([rng.uniform(0.1, 12, 1 << 16), rng.uniform(-6, 6, 1 << 12)]).astype(np.float32)
    b = np.concatenate([rng.uniform(0.1, 12, 1 << 16), rng.uniform(-6, 6, 1 << 12)]).astype(np.float32)
    ta, tb = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
    ob, ol = torch.empty_like(ta), torch.empty_like(ta)
    E.assign([ob, ol], [E.beta(E.Table(ta), E.Table(tb)), E.betaln(E.Table(ta), E.Table(tb))], precision=prec)
    got_b, got_l = ob.cpu().numpy(), ol.cpu().numpy()
    L = oracle.lib()
    want_b = np.float32([L.o_beta(float(p), float(q)) for p, q in zip(a, b)])
    want_l = np.float32([L.o_betaln(float(p), float(q)) for p, q in zip(a, b)])
    if prec == 1:
        assert _same(got_b, want_b).all() and _same(got_l, want_l).all()
    else:
        sp = pytest.importorskip("scipy.special")
        pos = (a > 0) & (b > 0)
        a64, b64 = a[pos].astype(np.float64), b[pos].astype(np.float64)
        terms = np.abs(sp.gammaln(a64)) + np.abs(sp.gammaln(b64)) + np.abs(sp.gammaln(a64 + b64))
        eps = float(np.finfo(np.float32).eps)
        assert np.max(np.abs(got_l[pos] - sp.betaln(a64, b64)) / terms) < 8 * eps
        rb = sp.beta(a64, b64)
        assert np.max(np.abs(got_b[pos] - rb) / np.abs(rb) / np.maximum(terms, 1.0)) < 16 * eps
        assert np.array_equal(np.isnan(got_b), np.isnan(want_b))
    for fn, out in (("beta", got_b), ("betaln", got_l)):
        rs = [r for r in golden if r["fn"] == fn]
        assert len(rs) >= 2
        tx = torch.tensor([r["x"] for r in rs], dtype=torch.float32, device=dev)
        ty = torch.tensor([r["y"] for r in rs], dtype=torch.float32, device=dev)
        o = torch.empty_like(tx)
        E.assign([o], [getattr(E, fn)(E.Table(tx), E.Table(ty))], precision=prec)
        for g, r in zip(o.cpu().numpy(), rs):
            assert nt2_ulpdist(g, r["expected"]) <= r["tol_nt2ulp"], (r, g)


@pytest.mark.parametrize("prec", [1, 0], ids=["nt2", "fast"])
def test_dawson_nthroot_expni(lib, dev, oracle, prec):
    """dawson (map and program), nthroot(x, n) and expni(n, x) (programs; the
    integer n carried in a float table): bit-identical to the oracle's
    restatement of NT2's float algorithms under the NT2 policy; under the fast
    one within a few ulp of FP64 (scipy's dawsn and expn, the double root) --
    dawson 4, nthroot 2 (or 1 more than NT2's own result where its Newton
    step's powers leave the normal range), expni 12 (NT2's own float expni
    reaches 10) -- with
    NT2's NaN positions; NT2's known answers (dawson.cpp, nthroot.cpp,
    expni.cpp) in both."""
    from nt2_gb300 import expr as E
    sp = pytest.importorskip("scipy.special")
    rng = np.random.default_rng(33)
    x = np.concatenate([rng.uniform(-12, 12, 1 << 16), np.exp(rng.uniform(-20, 25, 1 << 12)), SPECIALS,
                        -SPECIALS]).astype(np.float32)
    got = _run(lib, dev, "dawson", x, prec)
    tx = torch.from_numpy(x).to(dev)
    o = torch.empty_like(tx)
    E.assign([o], [E.dawson(E.Table(tx))], precision=prec)
    assert _same(o.cpu().numpy(), got).all()
    ref = oracle.map_f32("dawson", x)
    if prec == 1:
        assert _same(got, ref).all()
    else:
        r64 = sp.dawsn(x.astype(np.float64))
        ok = np.isfinite(r64) & (r64 != 0)
        assert (np.abs(got[ok] - r64[ok]) / np.spacing(np.abs(r64[ok]).astype(np.float32))).max() <= 4.0
        assert np.array_equal(np.isnan(got), np.isnan(ref))
    # nthroot: x over both signs and many scales, n in [-7, 7] (0 and the even
    # n of negative x included)
    xs = np.concatenate([rng.uniform(-50, 50, 1 << 15), np.exp(rng.uniform(-30, 30, 1 << 13)), SPECIALS,
                         -SPECIALS]).astype(np.float32)
    ns = rng.integers(-7, 8, xs.size).astype(np.float32)
    tx, tn = torch.from_numpy(xs).to(dev), torch.from_numpy(ns).to(dev)
    o = torch.empty_like(tx)
    E.assign([o], [E.nthroot(E.Table(tx), E.Table(tn))], precision=prec)
    got = o.cpu().numpy()
    ref = oracle.nthroot_f32(xs, ns)
    if prec == 1:
        assert _same(got, ref).all()
    else:
        assert np.array_equal(np.isnan(got), np.isnan(ref))
        ok = np.isfinite(ref) & (ref != 0) & (ns != 0)
        r64 = np.sign(xs[ok]).astype(np.float64) * np.abs(xs[ok].astype(np.float64)) ** (1.0 / ns[ok].astype(np.float64))
        sp32 = np.spacing(np.abs(r64).astype(np.float32))
        ulp, ulp_nt2 = np.abs(got[ok] - r64) / sp32, np.abs(ref[ok] - r64) / sp32
        # NT2's Newton step works on y^n and y^(n-1): where those leave the
        # normal range (|x| near the float limits) its own result drifts, and
        # the fast policy's with it
        bad = ulp > np.maximum(2.0, ulp_nt2 + 1.0)
        assert not bad.any(), (xs[ok][bad][:3], ns[ok][bad][:3], ulp[bad][:3], ulp_nt2[bad][:3])
    # expni: n in [0, 40] and 6000 (the large-n expansion), x in (0, 90]
    xe = np.concatenate([rng.uniform(0, 1, 1 << 13), rng.uniform(1, 90, 1 << 14), [0, -1, np.inf, np.nan]])
    ne = np.concatenate([rng.integers(0, 41, xe.size - 1024), np.full(1024, 6000)]).astype(np.float32)
    xe = xe.astype(np.float32)
    tx, tn = torch.from_numpy(xe).to(dev), torch.from_numpy(ne).to(dev)
    o = torch.empty_like(tx)
    E.assign([o], [E.expni(E.Table(tn), E.Table(tx))], precision=prec)
    got = o.cpu().numpy()
    ref = oracle.expni_f32(ne, xe)
    if prec == 1:
        assert _same(got, ref).all()
    else:
        assert np.array_equal(np.isnan(got), np.isnan(ref))
        r64 = sp.expn(ne.astype(np.int64), xe.astype(np.float64))
        ok = np.isfinite(r64) & (r64 > 1e-37) & np.isfinite(ref)
        ulp = np.abs(got[ok] - r64[ok]) / np.spacing(np.abs(r64[ok]).astype(np.float32))
        assert ulp.max() <= 12.0, (xe[ok][np.argmax(ulp)], ne[ok][np.argmax(ulp)], ulp.max())
    golden = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "nt2_unit_vectors.json")))
    rs = [r for r in golden if r["fn"] == "dawson"]
    for g, r in zip(_run(lib, dev, "dawson", np.float32([r["x"] for r in rs]), prec), rs):
        assert nt2_ulpdist(g, r["expected"]) <= r["tol_nt2ulp"], (r, g)
    for fn in ("nthroot", "expni"):
        rs = [r for r in golden if r["fn"] == fn]
        assert len(rs) >= 5
        ta = torch.tensor([r["x"] for r in rs], dtype=torch.float32, device=dev)
        tb = torch.tensor([r["y"] for r in rs], dtype=torch.float32, device=dev)
        o = torch.empty_like(ta)
        E.assign([o], [getattr(E, fn)(E.Table(ta), E.Table(tb))], precision=prec)
        for g, r in zip(o.cpu().numpy(), rs):
            assert nt2_ulpdist(g, r["expected"]) <= r["tol_nt2ulp"], (r, g)


@pytest.mark.parametrize("prec", [1, 0], ids=["nt2", "fast"])
def test_gammainc(lib, dev, prec):
    """gammainc(x, a) = P(a, x) (NT2 calls Boost.Math's gamma_p, which works
    in double for float arguments; this library's own double evaluation):
    within 1 ulp of scipy's FP64 value for a up to 1e4, within 1 ulp of the
    50-digit values of tests/golden/gammainc_large_a.json for a from 2e5 to
    1e9 (where scipy itself is off by up to 1e6 ulp), identical bits in both
    policies, NT2's special cases and known answers (gammainc.cpp)."""
    from nt2_gb300 import expr as E
    sp = pytest.importorskip("scipy.special")
    rng = np.random.default_rng(44)
    a = np.exp(rng.uniform(np.log(1e-3), np.log(1e4), 1 << 15))
    x = a * np.exp(rng.uniform(-3, 1.5, a.size))
    a = np.concatenate([a, [0, 0, 1, 1, 1, 1, 2, np.nan, -1, np.inf]]).astype(np.float32)
    x = np.concatenate([x, [5, np.inf, np.inf, 0, -0.0, np.nan, -1, 1, 1, 1]]).astype(np.float32)

    def run(xv, av, p):
        tx, ta = torch.from_numpy(xv).to(dev), torch.from_numpy(av).to(dev)
        o = torch.empty_like(tx)
        E.assign([o], [E.gammainc(E.Table(tx), E.Table(ta))], precision=p)
        return o.cpu().numpy()

    got = run(x, a, prec)
    assert _same(got, run(x, a, 1 - prec)).all()
    with np.errstate(invalid="ignore"):
        r64 = np.where((a == 0) | (x == np.inf), 1.0, sp.gammainc(a.astype(np.float64), x.astype(np.float64)))
    r64 = np.where(np.isnan(x) | np.isnan(a) | (x < 0) | (a < 0) | np.isinf(a), np.nan, r64)
    r64 = np.where((a == 0) | (x == np.inf), 1.0, r64)
    assert np.array_equal(np.isnan(got), np.isnan(r64))
    ok = np.isfinite(r64) & (r64 > 1e-37)
    ulp = np.abs(got[ok] - r64[ok]) / np.spacing(np.abs(r64[ok]).astype(np.float32))
    assert ulp.max() <= 1.0, (x[ok][np.argmax(ulp)], a[ok][np.argmax(ulp)], ulp.max())
    assert (np.abs(got[~ok & ~np.isnan(r64)]) <= np.float32(2e-37)).all()  # P underflows to 0 there
    big = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "gammainc_large_a.json")))
    g = run(np.float32([r["x"] for r in big]), np.float32([r["a"] for r in big]), prec)
    p = np.float64([r["p"] for r in big])
    keep = p > 1e-37
    assert (np.abs(g[keep] - p[keep]) / np.spacing(p[keep].astype(np.float32))).max() <= 1.0
    golden = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "nt2_unit_vectors.json")))
    rs = [r for r in golden if r["fn"] == "gammainc"]
    assert len(rs) >= 5
    for v, r in zip(run(np.float32([r["x"] for r in rs]), np.float32([r["y"] for r in rs]), prec), rs):
        assert nt2_ulpdist(v, r["expected"]) <= r["tol_nt2ulp"], (r, v)


@pytest.mark.parametrize("prec", [1, 0], ids=["nt2", "fast"])
def test_spence(lib, dev, oracle, prec):
    """spence (NT2's float dilogarithm, Cephes' coefficients): bit-identical to
    the oracle under the NT2 policy (map and program), within 6 ulp of FP64
    (scipy's spence; NT2's own float result reaches 4.5) under the fast one;
    NT2's known answers (spence.cpp) in both."""
    from nt2_gb300 import expr as E
    sp = pytest.importorskip("scipy.special")
    rng = np.random.default_rng(55)
    x = np.concatenate([rng.uniform(0, 3, 1 << 16), np.exp(rng.uniform(-30, 40, 1 << 13)), SPECIALS,
                        -SPECIALS]).astype(np.float32)
    got = _run(lib, dev, "spence", x, prec)
    tx = torch.from_numpy(x).to(dev)
    o = torch.empty_like(tx)
    E.assign([o], [E.spence(E.Table(tx))], precision=prec)
    assert _same(o.cpu().numpy(), got).all()
    ref = oracle.map_f32("spence", x)
    if prec == 1:
        assert _same(got, ref).all()
    else:
        assert np.array_equal(np.isnan(got), np.isnan(ref))
        with np.errstate(invalid="ignore"):
            r64 = sp.spence(x.astype(np.float64))
        ok = np.isfinite(r64) & (np.abs(r64) > 1e-30)
        ulp = np.abs(got[ok] - r64[ok]) / np.spacing(np.abs(r64[ok]).astype(np.float32))
        assert ulp.max() <= 6.0, (x[ok][np.argmax(ulp)], ulp.max())
    golden = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "nt2_unit_vectors.json")))
    rs = [r for r in golden if r["fn"] == "spence"]
    assert len(rs) >= 5
    for g, r in zip(_run(lib, dev, "spence", np.float32([r["x"] for r in rs]), prec), rs):
        assert nt2_ulpdist(g, r["expected"]) <= r["tol_nt2ulp"], (r, g)


@pytest.mark.parametrize("prec", [1, 0], ids=["nt2", "fast"])
def test_gammaincinv_and_stirling(lib, dev, oracle, prec):
    """gammaincinv(p, a), the x with P(a, x) = p (NT2 calls Boost.Math's
    gamma_p_inv, in double for float arguments; this library's own double
    Halley iteration): within 1 ulp of scipy's FP64 inverse for a up to 1e4,
    gammainc(gammaincinv(p, a), a) back within 2 ulp of p where P is not flat,
    identical bits in both policies, NT2's known answers (gammaincinv.cpp).
    stirling (NT2's Stirling approximation of Gamma): bit-identical to the
    oracle under the NT2 policy; under the fast one no more than 4 ulp beyond
    NT2's own distance from the same formula in FP64; NT2's known answers
    (stirling.cpp)."""
    from nt2_gb300 import expr as E
    sp = pytest.importorskip("scipy.special")
    rng = np.random.default_rng(66)
    a = np.exp(rng.uniform(np.log(1e-2), np.log(1e4), 1 << 14)).astype(np.float32)
    p = rng.uniform(0, 1, a.size).astype(np.float32)
    p[:64] = np.float32([0, 1, np.nan, -0.5, 1.5] + [1e-30] * 59)
    ta, tp = torch.from_numpy(a).to(dev), torch.from_numpy(p).to(dev)

    def run(e, q):
        o = torch.empty_like(ta)
        E.assign([o], [e], precision=q)
        return o.cpu().numpy()

    got = run(E.gammaincinv(E.Table(tp), E.Table(ta)), prec)
    assert _same(got, run(E.gammaincinv(E.Table(tp), E.Table(ta)), 1 - prec)).all()
    with np.errstate(invalid="ignore"):
        r64 = sp.gammaincinv(a.astype(np.float64), p.astype(np.float64))
    r64 = np.where(p == 1, np.inf, np.where(np.isnan(p) | (p < 0) | (p > 1), np.nan, r64))
    assert np.array_equal(np.isnan(got), np.isnan(r64))
    ok = np.isfinite(r64) & (r64 > 1e-37)
    ulp = np.abs(got[ok] - r64[ok]) / np.spacing(r64[ok].astype(np.float32))
    assert ulp.max() <= 1.0, (a[ok][np.argmax(ulp)], p[ok][np.argmax(ulp)], ulp.max())
    back = run(E.gammainc(E.Table(torch.from_numpy(got).to(dev)), E.Table(ta)), prec)
    fin = np.isfinite(got) & (got > 1e-30) & (p > 1e-6) & (p < 1 - 1e-6)
    # |dP/dx| * spacing(x) bounds how far P moves between neighbouring floats of x
    dpdx = np.exp((a[fin].astype(np.float64) - 1) * np.log(got[fin].astype(np.float64)) - got[fin] - sp.gammaln(a[fin].astype(np.float64)))
    slack = dpdx * np.spacing(got[fin]) + 2 * np.spacing(p[fin])
    assert (np.abs(back[fin].astype(np.float64) - p[fin]) <= slack).all()
    golden = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "nt2_unit_vectors.json")))
    rs = [r for r in golden if r["fn"] == "gammaincinv"]
    assert len(rs) >= 4
    tx = torch.tensor([r["x"] for r in rs], dtype=torch.float32, device=dev)
    ty = torch.tensor([r["y"] for r in rs], dtype=torch.float32, device=dev)
    o = torch.empty_like(tx)
    E.assign([o], [E.gammaincinv(E.Table(tx), E.Table(ty))], precision=prec)
    for v, r in zip(o.cpu().numpy(), rs):
        assert nt2_ulpdist(v, r["expected"]) <= r["tol_nt2ulp"], (r, v)
    # stirling
    x = np.concatenate([rng.uniform(0.5, 36, 1 << 15), SPECIALS, -SPECIALS]).astype(np.float32)
    got = _run(lib, dev, "stirling", x, prec)
    ref = oracle.map_f32("stirling", x)
    if prec == 1:
        assert _same(got, ref).all()
    else:
        assert np.array_equal(np.isnan(got), np.isnan(ref))
        c = np.float32([np.uint32(v).view(np.float32) for v in (0xb970b359, 0xbb2fb930, 0x3b638e39, 0x3daaaaab)])
        x64 = x.astype(np.float64)
        with np.errstate(all="ignore"):
            w = 1.0 / x64
            w = w * (((c[0] * w + c[1]) * w + c[2]) * w + c[3]) + 1.0
            f64 = np.sqrt(2 * np.pi) * w * np.exp(-x64) * x64 ** (x64 - 0.5)
        ok = np.isfinite(f64) & (f64 > 1e-30) & np.isfinite(ref) & (x > 0)
        sp32 = np.spacing(f64[ok].astype(np.float32))
        e_fast, e_nt2 = np.abs(got[ok] - f64[ok]) / sp32, np.abs(ref[ok] - f64[ok]) / sp32
        assert (e_fast <= e_nt2 + 4.0).all(), (x[ok][np.argmax(e_fast - e_nt2)], (e_fast - e_nt2).max())
    rs = [r for r in golden if r["fn"] == "stirling"]
    assert len(rs) >= 4
    for g, r in zip(_run(lib, dev, "stirling", np.float32([r["x"] for r in rs]), prec), rs):
        assert nt2_ulpdist(g, r["expected"]) <= r["tol_nt2ulp"], (r, g)
