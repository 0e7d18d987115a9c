"""Reverse mode of any program (nt2g_program_vjp) against FP64.

References:
  - FP64 forward-mode dual numbers over the same expression (tests/helpers.py:
    Dual), themselves checked here against FP64 central differences;
  - the oracle's FP64 analytic Black-Scholes VJP (the one the fused adjoint
    kernel is held to) for the textbook form;
  - central differences of the GPU's own float forward (loose: float rounding
    over the step);
  - per opcode, FP64 central differences of the function (numpy / scipy).

Gradient errors are measured against the gradient's term scale -- the sum
over the expression's paths of |product of local partials| times |cotangent|
-- which is the gradient's own magnitude except where the chain-rule terms
cancel; floor 2^-100 (below it FP32 holds the terms only as subnormals).
The demo form (demo/blackscholes/nt2/blackandscholes_nt2.cpp:55-59) uses NT2's
fastnormcdf, whose derivative here is that of the approximation itself."""
import zlib

import numpy as np
import pytest
import torch

from helpers import Dual, bs_demo_dual, d_abs, d_exp, d_log1p, d_sqr, d_sqrt, fastnormcdf64
from nt2_gb300 import expr as E

pytestmark = pytest.mark.gpu

F32 = np.float32
SCALE_FLOOR = 2.0 ** -100
TERM_TOL = 2e-6  # |error| / term scale; the fused Black-Scholes adjoint is held to 1e-5
TEXTBOOK_TOL = 5e-6  # normcdf of a computed d1 (|d1| up to ~6 above the floors): d1^2 ulp


def _t(dev, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _demo_inputs(n, seed=1006):
    rng = np.random.default_rng(seed)
    return (rng.uniform(5, 30, n).astype(F32), rng.uniform(1, 100, n).astype(F32),
            rng.uniform(0.25, 10, n).astype(F32), rng.uniform(0.01, 0.05, n).astype(F32),
            rng.uniform(0.1, 0.6, n).astype(F32), rng.uniform(-1, 1, n).astype(F32))


def _demo_expr(S, X, T, r, v):
    da = E.sqrt(T)
    d1 = E.log(S / X) + (E.fma(E.sqr(v), 0.5, r) * T) / (v * da)
    d2 = E.fnms(v, da, d1)
    return E.fnms(X * E.exp(-r * T), E.fastnormcdf(d2), S * E.fastnormcdf(d1))


def _term_err(got, ref, scale):
    return np.abs(np.asarray(got, np.float64) - ref) / np.maximum(scale, SCALE_FLOOR)


def test_dual_reference_matches_fp64_central_differences():
    """The FP64 reference itself: dual-number gradients of the demo form
    against FP64 central differences (step 1e-6 relative)."""
    S, X, T, r, v, _ = (a.astype(np.float64) for a in _demo_inputs(4096))
    base = [S, X, T, r, v]
    R = bs_demo_dual(*[Dual.var(a, i, 5) for i, a in enumerate(base)])
    f = lambda *a: bs_demo_dual(*[Dual.var(x, 0, 1) for x in a]).v  # noqa: E731
    for i in range(5):
        h = 1e-6 * np.maximum(1.0, np.abs(base[i]))
        p, m = list(base), list(base)
        p[i], m[i] = base[i] + h, base[i] - h
        fd = (f(*p) - f(*m)) / (2 * h)
        assert _term_err(fd, R.t[i], R.a[i]).max() < 1e-6, i


@pytest.mark.parametrize("prec", ["fast", "nt2"])
def test_demo_bs_tables_against_fp64(lib, dev, prec):
    """Every input of the demo form a table (2^20 options + 3): each gradient
    table within TERM_TOL of the FP64 dual-number VJP, relative to its term
    scale; the cotangent's output table is not written."""
    p = lib.PREC_NT2 if prec == "nt2" else lib.PREC_FAST
    n = (1 << 20) + 3
    S, X, T, r, v, gR = _demo_inputs(n)
    t = [_t(dev, a) for a in (S, X, T, r, v)]
    R = torch.full((n,), 7.0, device=dev)
    grads = E.vjp([R], [_demo_expr(*[E.Table(x) for x in t])], [_t(dev, gR)], t, precision=p)
    torch.cuda.synchronize()
    assert bool((R == 7.0).all())
    ref = bs_demo_dual(*[Dual.var(a.astype(np.float64), i, 5) for i, a in enumerate((S, X, T, r, v))])
    g64 = gR.astype(np.float64)
    for i, name in enumerate(["dS", "dX", "dT", "dr", "dv"]):
        e = _term_err(grads[i].cpu().numpy(), g64 * ref.t[i], np.abs(g64) * ref.a[i])
        print(f"\n{prec} {name}: max {e.max():.3e} mean {e.mean():.3e} (term scale)")
        assert e.max() <= TERM_TOL, (name, e.max())


def test_demo_bs_scalars_summed_and_deterministic(lib, dev):
    """r and v as scalars (the demo's r, v as one number each): their
    gradients are the per-option gradients summed over 2^22 options, within
    TERM_TOL of the FP64 sum relative to the summed term scales, and the same
    bits on a second run."""
    n = 1 << 22
    S, X, T, r, v, gR = _demo_inputs(n, seed=1007)
    r0, v0 = 0.03, 0.35
    t = [_t(dev, a) for a in (S, X, T)]
    rs, vs = E.Scalar(r0), E.Scalar(v0)
    R = torch.empty(n, device=dev)
    ct = _t(dev, gR)

    def run():
        return E.vjp([R], [_demo_expr(E.Table(t[0]), E.Table(t[1]), E.Table(t[2]), rs, vs)], [ct],
                     [t[0], rs, vs])

    g1 = run()
    g2 = run()
    torch.cuda.synchronize()
    # gradients of (S, r, v) along three directions; X, T constants
    d = [Dual.var(S.astype(np.float64), 0, 3)]
    zero = lambda a: Dual(np.asarray(a, np.float64), np.zeros((3, n)), np.zeros((3, n)))  # noqa: E731
    rr = Dual(np.full(n, float(np.float32(r0))), np.zeros((3, n)), np.zeros((3, n)))
    rr.t[1] = rr.a[1] = 1.0
    vv = Dual(np.full(n, float(np.float32(v0))), np.zeros((3, n)), np.zeros((3, n)))
    vv.t[2] = vv.a[2] = 1.0
    ref = bs_demo_dual(d[0], zero(X), zero(T), rr, vv)
    g64 = gR.astype(np.float64)
    e = _term_err(g1[0].cpu().numpy(), g64 * ref.t[0], np.abs(g64) * ref.a[0])
    assert e.max() <= TERM_TOL
    for k, name in ((1, "dr"), (2, "dv")):
        exact = float(np.sum(g64 * ref.t[k]))
        scale = float(np.sum(np.abs(g64) * ref.a[k]))
        got = float(g1[k].item())
        print(f"\n{name}: sum {got:.10g} exact {exact:.10g} err/scale {abs(got - exact) / scale:.3e}")
        assert abs(got - exact) <= TERM_TOL * scale
        assert float(g2[k].item()) == got  # deterministic


def test_demo_bs_against_gpu_central_differences(lib, dev):
    """The VJP with a unit cotangent against central differences of the GPU's
    own float forward (nt2g_eval of the same program), Richardson-extrapolated
    (4 D(h/2) - D(h)) / 3 with h = 2^-7 of the input: |VJP - quotient| within
    1e-2 of the term scale (the quotient's truncation) plus the float forward's
    rounding over the steps (4 ulp of max(S, X) per evaluation, through the
    extrapolation) -- the quotient's own error; the FP64 tests above hold the
    gradients to TERM_TOL."""
    n = 8192
    S, X, T, r, v, _ = _demo_inputs(n, seed=1008)
    base = [S, X, T, r, v]
    t = [_t(dev, a) for a in base]
    one = torch.ones(n, device=dev)
    R = torch.empty(n, device=dev)
    grads = E.vjp([R], [_demo_expr(*[E.Table(x) for x in t])], [one], t)
    ref = bs_demo_dual(*[Dual.var(a.astype(np.float64), i, 5) for i, a in enumerate(base)])

    def forward(i, xi):
        xs = list(t)
        xs[i] = _t(dev, xi)
        o = torch.empty(n, device=dev)
        E.assign([o], [_demo_expr(*[E.Table(x) for x in xs])], force_generic=1)
        return o.cpu().numpy().astype(np.float64)

    # R = S N(d1) - X e^-rT N(d2): its float rounding is relative to the terms, at most max(S, X)
    ulp_terms = np.spacing(np.maximum(S, X)).astype(np.float64)

    def quotient(i, h):
        up, dn = (base[i] + h).astype(F32), (base[i] - h).astype(F32)
        step = up.astype(np.float64) - dn.astype(np.float64)
        return (forward(i, up) - forward(i, dn)) / step, ulp_terms / step

    for i in range(5):
        h = (np.float32(2.0 ** -7) * np.abs(base[i])).astype(F32)
        d1, u1 = quotient(i, h)
        d2, u2 = quotient(i, (h / 2).astype(F32))
        fd = (4 * d2 - d1) / 3
        noise = 4 * (4 * u2 + u1) / 3  # 4 ulp of the terms per evaluation, through the extrapolation
        err = np.abs(grads[i].cpu().numpy().astype(np.float64) - fd)
        print(f"\ninput {i}: GPU central differences vs VJP, max {(err / ref.a[i]).max():.3e} of term scale, "
              f"max {(err / (1e-2 * ref.a[i] + noise)).max():.3f} of the bound")
        assert np.all(err <= 1e-2 * ref.a[i] + noise), i


def test_textbook_bs_against_oracle_vjp(lib, dev, oracle):
    """The textbook Black-Scholes (normcdf, sigma a table, r a scalar) through
    the program VJP against the oracle's FP64 analytic VJP -- the reference of
    the fused adjoint kernel; dr is the sum over the options.  The term scale
    is the program's own (FP64 duals over the same expression): the chain rule
    carries S phi(d1) dd1 and K e^-rT phi(d2) dd2 as separate terms, which the
    analytic formula cancels (S phi(d1) = K e^-rT phi(d2)) before it adds.
    Bound TEXTBOOK_TOL, with the fused kernel's natural floors (1e-10 of
    (|gc| + |gp|) times 1, 1, S, S sqrt(T)): the float forward's rounding of
    d1 is magnified d1^2 times in phi(d1), which the generic chain rule, fed
    the forward's float values, inherits; the fused adjoint kernel carries
    d1's residual (measured max 1.7e-6 here, over 2^20 options)."""
    from helpers import bs_textbook_dual
    from helpers import bs_inputs
    n = 1 << 20
    S, K, T, sig = bs_inputs(n, seed=1004, sigma_table=True)
    rng = np.random.default_rng(1005)
    gc, gp = rng.uniform(-1, 1, n).astype(F32), rng.uniform(-1, 1, n).astype(F32)
    r = 0.02
    t = [_t(dev, a) for a in (S, K, T, sig)]
    St, Kt, Tt, st = (E.Table(x) for x in t)
    rs = E.Scalar(r)
    sq = E.sqrt(Tt)
    d1 = (E.log(St / Kt) + E.fma(E.sqr(st), 0.5, rs) * Tt) / (st * sq)
    d2 = E.fnms(st, sq, d1)
    e = Kt * E.exp(-rs * Tt)
    C, P = torch.empty(n, device=dev), torch.empty(n, device=dev)
    grads = E.vjp([C, P], [E.fnms(e, E.normcdf(d2), St * E.normcdf(d1)), E.fnms(St, E.normcdf(-d1),
                                                                                e * E.normcdf(-d2))],
                  [_t(dev, gc), _t(dev, gp)], t + [rs])
    torch.cuda.synchronize()
    ref = oracle.blackscholes_vjp_f64(S, K, T, sig, r, gc, gp)
    rr = Dual(np.full(n, float(np.float32(r))), np.zeros((5, n)), np.zeros((5, n)))
    rr.t[4] = rr.a[4] = 1.0
    c, p = bs_textbook_dual(*[Dual.var(a.astype(np.float64), i, 5) for i, a in enumerate((S, K, T, sig))], rr)
    g1, g2 = gc.astype(np.float64), gp.astype(np.float64)
    g, s64, k64, t64 = np.abs(g1) + np.abs(g2), S.astype(np.float64), K.astype(np.float64), T.astype(np.float64)
    floors = [1e-10 * g * x for x in (np.ones(n), np.ones(n), s64, s64 * np.sqrt(t64))]
    for i, name in enumerate(["dS", "dK", "dT", "dsigma", "dr"]):
        scale = np.abs(g1) * c.a[i] + np.abs(g2) * p.a[i]
        dual = g1 * c.t[i] + g2 * p.t[i]
        assert _term_err(dual, ref[i], scale).max() < 1e-9  # the two FP64 references agree
        if i < 4:
            err = _term_err(grads[i].cpu().numpy(), ref[i], np.maximum(scale, floors[i]))
            print(f"\n{name}: max {err.max():.3e} mean {err.mean():.3e} (term scale)")
            assert err.max() <= TEXTBOOK_TOL, name
        else:
            exact, sc = float(np.sum(ref[4])), float(np.sum(scale))
            assert abs(float(grads[4].item()) - exact) <= TERM_TOL * sc


def test_expr3_against_analytic(lib, dev):
    """exp(-x^2) sqrt|y| + log1p|z| (the library's expr3): closed-form FP64
    gradients; in-place gradient tables (each gradient written over its own
    input) give the same bits."""
    n = (1 << 20) + 1
    rng = np.random.default_rng(1009)
    x, y, z = (rng.standard_normal(n).astype(F32) for _ in range(3))
    g = rng.uniform(-1, 1, n).astype(F32)
    t = [_t(dev, a) for a in (x, y, z)]
    out = torch.empty(n, device=dev)

    def expr(a, b, c):
        return E.exp(-E.sqr(a)) * E.sqrt(E.abs_(b)) + E.log1p(E.abs_(c))

    grads = E.vjp([out], [expr(*[E.Table(q) for q in t])], [_t(dev, g)], t)
    ds = [Dual.var(a.astype(np.float64), i, 3) for i, a in enumerate((x, y, z))]
    ref = d_exp(-d_sqr(ds[0])) * d_sqrt(d_abs(ds[1])) + d_log1p(d_abs(ds[2]))
    g64 = g.astype(np.float64)
    for i in range(3):
        e = _term_err(grads[i].cpu().numpy(), g64 * ref.t[i], np.abs(g64) * ref.a[i])
        print(f"\nexpr3 d{'xyz'[i]}: max {e.max():.3e} (term scale)")
        assert e.max() <= TERM_TOL
    # gradients written over the inputs themselves
    ti = [q.clone() for q in t]
    prog, slots = E.compile_program([out], [expr(*[E.Table(q) for q in ti])])
    import ctypes
    args, cnt = E._args_of(slots)
    ns = len(slots)
    ct, tg = (ctypes.c_void_p * ns)(), (ctypes.c_void_p * ns)()
    gt = _t(dev, g)
    ct[E._slot_of(slots, out)] = gt.data_ptr()
    for q in ti:
        tg[E._slot_of(slots, q)] = q.data_ptr()
    lib.check(lib.load().nt2g_program_vjp(prog.handle, args, ns, cnt, ct, tg, None, 0, None, 0, lib._stream()))
    torch.cuda.synchronize()
    for a, b in zip(ti, grads):
        assert torch.equal(a.view(torch.int32), b.view(torch.int32))


# (E function, FP64 reference, domain low, domain high, signed domain)
def _unary_cases():
    from scipy import special as sp
    pi = np.pi
    rad = pi / 180
    return {
        "exp": (np.exp, -5, 5), "log": (np.log, 0.1, 10), "log1p": (np.log1p, -0.5, 5), "expm1": (np.expm1, -3, 3),
        "exp2": (np.exp2, -5, 5), "exp10": (lambda x: 10.0 ** x, -2, 2), "log2": (np.log2, 0.1, 10),
        "log10": (np.log10, 0.1, 10), "sin": (np.sin, -10, 10), "cos": (np.cos, -10, 10), "tan": (np.tan, -1.2, 1.2),
        "sinpi": (lambda x: np.sin(pi * x), -3, 3), "cospi": (lambda x: np.cos(pi * x), -3, 3),
        "tanpi": (lambda x: np.tan(pi * x), -0.4, 0.4),
        "proper_tanpi": (lambda x: np.tan(pi * x), -0.45, 0.45), "cot": (lambda x: 1 / np.tan(x), 0.2, 2.9),
        "sec": (lambda x: 1 / np.cos(x), -1.2, 1.2), "csc": (lambda x: 1 / np.sin(x), 0.3, 2.8),
        "cotpi": (lambda x: 1 / np.tan(pi * x), 0.1, 0.9), "secpi": (lambda x: 1 / np.cos(pi * x), -0.4, 0.4),
        "cscpi": (lambda x: 1 / np.sin(pi * x), 0.1, 0.9), "sind": (lambda x: np.sin(rad * x), -400, 400),
        "cosd": (lambda x: np.cos(rad * x), -400, 400), "tand": (lambda x: np.tan(rad * x), -70, 70),
        "cotd": (lambda x: 1 / np.tan(rad * x), 10, 170), "secd": (lambda x: 1 / np.cos(rad * x), -70, 70),
        "cscd": (lambda x: 1 / np.sin(rad * x), 10, 170), "sinc": (lambda x: np.sin(x) / x, -10, 10),
        "sincpi": (lambda x: np.sin(pi * x) / (pi * x), -3, 3), "sinh": (np.sinh, -5, 5), "cosh": (np.cosh, -5, 5),
        "tanh": (np.tanh, -3, 3), "coth": (lambda x: 1 / np.tanh(x), 0.2, 3), "sinhc": (lambda x: np.sinh(x) / x, -5, 5),
        "asin": (np.arcsin, -0.9, 0.9), "acos": (np.arccos, -0.9, 0.9), "atan": (np.arctan, -10, 10),
        "asinh": (np.arcsinh, -10, 10), "acosh": (np.arccosh, 1.1, 10), "atanh": (np.arctanh, -0.9, 0.9),
        "acotd": (lambda x: np.degrees(np.arctan(1 / x)), 0.1, 10), "asec": (lambda x: np.arccos(1 / x), 1.1, 10),
        "acsc": (lambda x: np.arcsin(1 / x), 1.1, 10), "asech": (lambda x: np.arccosh(1 / x), 0.05, 0.95),
        "acoth": (lambda x: np.arctanh(1 / x), 1.1, 10), "acsch": (lambda x: np.arcsinh(1 / x), 0.1, 10),
        "cbrt": (np.cbrt, 0.1, 10), "sqrt": (np.sqrt, 0.1, 10), "sqr": (np.square, -5, 5),
        "rec": (lambda x: 1 / x, 0.1, 10), "abs_": (np.abs, 0.1, 5), "erf": (sp.erf, -3, 3), "erfc": (sp.erfc, -3, 3),
        "erfcx": (sp.erfcx, -1, 5), "expx2": (lambda x: np.exp(x * x), -3, 3), "gamma": (sp.gamma, 0.2, 5),
        "gammaln": (sp.gammaln, 0.2, 10), "erfinv": (sp.erfinv, -0.9, 0.9), "erfcinv": (sp.erfcinv, 0.1, 1.9),
        "exprecneg": (lambda x: np.exp(-1 / x), 0.2, 5), "exprecnegc": (lambda x: 1 - np.exp(-1 / x), 0.2, 5),
        "sqrt1pm1": (lambda x: np.sqrt(1 + x) - 1, -0.5, 5), "normcdf": (sp.ndtr, -5, 5),
        "fastnormcdf": (lambda x: fastnormcdf64(x)[0], -5, 5), "frac": (lambda x: x - np.trunc(x), -10, 10),
        "dawson": (sp.dawsn, -6, 6), "spence": (sp.spence, 0.05, 4),
    }


SIGNED = {"abs_", "cbrt", "rec", "acotd", "asec", "acsc", "acoth", "acsch", "coth"}
UNARY_TOL = 4e-6  # |error| / (|derivative| + floor), away from each function's singularities
# erfcx' = 2x erfcx(x) - 2/sqrt(pi) cancels as x grows: erfcx's own rounding
# is magnified ~x^2 times (2e-5 at x = 5); dawson' = 1 - 2x D(x) cancels to
# zero at D's maximum (|x| = 0.924), where one rounding of 1 is 1.2e-5 of the
# floor
UNARY_TOL_OF = {"erfcx": 2e-5, "dawson": 2e-5}


def _floor(name, x64, ref):
    """Where the derivative passes through zero its size is no measure of the
    rounding of the terms that make it: 1e-2 of its largest magnitude over the
    domain, and for gamma / gammaln the scale of digamma's terms (Gamma(x)
    (|ln x| + 1), |ln x| + 1)."""
    from scipy import special as sp
    if name == "gamma":
        return np.abs(sp.gamma(x64)) * (np.abs(np.log(x64)) + 1.0)
    if name == "gammaln":
        return np.abs(np.log(x64)) + 1.0
    return 1e-2 * np.max(np.abs(ref))


def _fd64(f64, x64):
    """FP64 central differences, Richardson-extrapolated (4 D(h/2) - D(h)) / 3
    with h = 2e-4 max(1, |x|): truncation O(h^4), rounding ~1e-12 |f|."""
    h = 2e-4 * np.maximum(1.0, np.abs(x64))
    d = lambda s: (f64(x64 + s) - f64(x64 - s)) / (2 * s)  # noqa: E731
    return (4 * d(h / 2) - d(h)) / 3


@pytest.mark.parametrize("name", sorted(_unary_cases()))
def test_unary_rule_against_fp64_central_differences(lib, dev, name):
    """Each unary opcode's adjoint rule: d op(x)/dx from the VJP with a unit
    cotangent, against FP64 central differences of the function, on 4096
    points of a domain inside its smooth range (both signs where the domain is
    symmetric under negation); relative error against |derivative| plus a
    floor for the derivative's zeros."""
    f64, lo, hi = _unary_cases()[name]
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    x = rng.uniform(lo, hi, 4096).astype(F32)
    if name in SIGNED:
        x = np.where(rng.random(4096) < 0.5, -x, x).astype(F32)
    if name == "fastnormcdf":  # NT2's approximation has a jump in its second derivative at 0
        x = x[np.abs(x) > 1e-2]
    if name == "frac":
        x = x[np.abs(x - np.round(x)) > 1e-2]  # the difference quotient's steps stay off the jumps
    tx = _t(dev, x)
    out = torch.empty_like(tx)
    (g,) = E.vjp([out], [getattr(E, name)(E.Table(tx))], [torch.ones_like(tx)], [tx])
    x64 = x.astype(np.float64)
    ref = _fd64(f64, x64)
    got = g.cpu().numpy().astype(np.float64)
    rel = np.abs(got - ref) / (np.abs(ref) + _floor(name, x64, ref))
    print(f"\n{name}: max rel err {rel.max():.3e}")
    assert rel.max() <= UNARY_TOL_OF.get(name, UNARY_TOL), (name, rel.max(), x[np.argmax(rel)])


def test_binary_and_select_rules(lib, dev):
    """pow, atan2, hypot, division, min, max, copysign, fma, fnms, if_else,
    selinc, seldec: both (all three) operands' gradients against FP64 central
    differences; piecewise-constant operations pass no gradient."""
    from scipy import special as sp
    n = 4096
    rng = np.random.default_rng(1010)
    x = rng.uniform(0.5, 3, n).astype(F32)
    y = rng.uniform(-2, 2, n).astype(F32)
    y = np.where(np.abs(y) < 0.05, F32(0.7), y).astype(F32)  # off 0 and off round()'s jumps
    z = rng.uniform(-3, 3, n).astype(F32)
    z = np.where(np.abs(z - y) < 1e-2, z + F32(0.1), z).astype(F32)
    cases = [
        (lambda a, b, c: E.pow(a, b), lambda a, b, c: a ** b),
        (lambda a, b, c: E.atan2(b, c), lambda a, b, c: np.arctan2(b, c)),
        (lambda a, b, c: E.hypot(b, c), lambda a, b, c: np.hypot(b, c)),
        (lambda a, b, c: b / a, lambda a, b, c: b / a),
        (lambda a, b, c: E.min_(b, c) + E.max_(b, c) * 2.0, lambda a, b, c: np.minimum(b, c) + 2 * np.maximum(b, c)),
        (lambda a, b, c: E.copysign(b, c) * a, lambda a, b, c: np.copysign(b, c) * a),
        (lambda a, b, c: E.fma(a, b, c) - E.fnms(b, c, a), lambda a, b, c: a * b + c - (a - b * c)),
        (lambda a, b, c: E.if_else(b > c, a * b, c) + E.selinc(a > 1.0, c) + E.seldec(a < 2.0, b),
         lambda a, b, c: np.where(b > c, a * b, c) + np.where(a > 1, c + 1, c) + np.where(a < 2, b - 1, b)),
        (lambda a, b, c: E.floor(a) * b + E.sign(c) + E.round(b),
         lambda a, b, c: np.floor(a) * b + np.sign(c) + np.round(b)),
        # integer operands (n) pass no gradient; gammainc's rule is for x only.
        # One function a case: a sum of them would cross zero, where the
        # terms' own rounding is no longer small against the 1e-3 floor
        (lambda a, b, c: E.nthroot(a, 3.0) * b, lambda a, b, c: np.cbrt(a) * b),
        (lambda a, b, c: E.nthroot(a, -2.0), lambda a, b, c: a ** -0.5),
        (lambda a, b, c: E.expni(2.0, a), lambda a, b, c: sp.expn(2, a)),
        (lambda a, b, c: E.expni(0.0, a), lambda a, b, c: sp.expn(0, a)),
        (lambda a, b, c: E.gammainc(a, 2.5), lambda a, b, c: sp.gammainc(2.5, a)),
    ]
    ins = [x, y, z]
    t = [_t(dev, a) for a in ins]
    for k, (fe, f64) in enumerate(cases):
        out = torch.empty(n, device=dev)
        grads = E.vjp([out], [fe(*[E.Table(q) for q in t])], [torch.ones(n, device=dev)], t)
        base = [a.astype(np.float64) for a in ins]
        for i in range(3):  # plain central differences: a small step keeps clear of the jumps
            h = 1e-6 * np.maximum(1.0, np.abs(base[i]))
            p, m = list(base), list(base)
            p[i], m[i] = base[i] + h, base[i] - h
            ref = (f64(*p) - f64(*m)) / (2 * h)
            got = grads[i].cpu().numpy().astype(np.float64)
            rel = np.abs(got - ref) / (np.abs(ref) + 1e-3)
            assert rel.max() <= UNARY_TOL, (k, i, rel.max())
