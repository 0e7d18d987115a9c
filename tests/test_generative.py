"""Generative leaves (colon / _, linspace, logspace).

CPU: the oracle's restatement against the known answers of NT2's own
generative unit tests (modules/core/generative/unit/table/{colon,linspace,
logspace}.cpp) and the Python mirror's element counts against the oracle's.
GPU: the INDEX leaf through the interpreter and the compiled kernel, bit-exact
under NT2's policy, absolute positions for partial ranges, p > 2^24 rounding,
uint8 wrap-around, and generative leaves inside larger expressions.
"""
import numpy as np
import pytest
import torch

from helpers import nt2_ulpdist
from nt2_gb300 import expr as E
from nt2_gb300 import lib as L

f = np.float32
PI = np.uint32(0x40490fdb).view(np.float32)
LOG10_PI = np.uint32(0x3efe8a6e).view(np.float32)


def _max_ulp(a, b):
    return max((nt2_ulpdist(x, y) for x, y in zip(a, b)), default=0.0)


def test_colon_known_answers(oracle):
    # colon.cpp:54-62: _(9, 0) is empty; :64-77: _(0, 9) = 0..9
    assert oracle.colon_nt2(9, 0).size == 0
    assert np.array_equal(oracle.colon_nt2(0, 9), np.arange(10, dtype=np.float32))
    # colon.cpp:136-164: real steps, refs written as T(l) + T(s)*T(i-1)
    x = oracle.colon_nt2(0, 0.3, 1)
    assert x.size == 4 and _max_ulp(x, [f(0) + f(0.3) * f(i) for i in range(4)]) <= 0.5
    y = oracle.colon_nt2(1, -0.3, 0)
    assert y.size == 4 and _max_ulp(y, [f(1) + f(-0.3) * f(i) for i in range(4)]) <= 2
    z = oracle.colon_nt2(0.5, 0, 6)
    assert z.size == 6 and (z == f(0.5)).all()


def test_linspace_known_answers(oracle):
    # linspace.cpp:56-79: 100 points by default, refs T(l) + (T(u-l)/99)*(i-1), 15 NT2 ulps
    x = oracle.linspace_nt2(0, 1)
    assert x.size == 100 and _max_ulp(x, [f(0) + (f(1) / f(99)) * f(i) for i in range(100)]) <= 15
    xr = oracle.linspace_nt2(1, 0)
    assert _max_ulp(xr, [f(1) + (f(-1) / f(99)) * f(i) for i in range(100)]) <= 15
    # :81-107: 7 points, 1 ulp; n = 1 gives the upper bound
    x7 = oracle.linspace_nt2(0, 1, 7)
    assert x7.size == 7 and _max_ulp(x7, [f(0) + (f(1) / f(6)) * f(i) for i in range(7)]) <= 1
    assert _max_ulp(oracle.linspace_nt2(1, 0, 7), [f(1) + (f(-1) / f(6)) * f(i) for i in range(7)]) <= 1
    assert np.array_equal(oracle.linspace_nt2(0, 9, 1), [9])
    # :109-120: no zero from -100 up to the float before 0
    for i in range(8):
        assert (oracle.linspace_nt2(-100, -1.4e-45, 100 + i) != 0).all()
    # :122-131: linspace(-1, 1, 257) hits -1 + k/128 exactly
    assert np.array_equal(oracle.linspace_nt2(-1, 1, 257), [f(-1) + f(k) / f(128) for k in range(257)])


def test_logspace_known_answers(oracle):
    # logspace.cpp:53-92: exp10(linspace(l, u, n)) within 1 NT2 ulp, 50 points by default
    for n, (lo, hi) in ((50, (0, 1)), (50, (1, 0)), (7, (0, 1)), (7, (1, 0))):
        x = oracle.logspace_nt2(lo, hi) if n == 50 else oracle.logspace_nt2(lo, hi, n)
        assert x.size == n and _max_ulp(x, oracle.map_f32("exp10", oracle.linspace_nt2(lo, hi, n))) <= 1
    # :95-115: u == pi means log10(pi) unless regular
    x = oracle.logspace_nt2(2, PI, 7)
    assert _max_ulp(x, oracle.map_f32("exp10", oracle.linspace_nt2(2, LOG10_PI, 7))) <= 1
    xr = oracle.logspace_nt2(2, PI, 7, regular=True)
    assert _max_ulp(xr, oracle.map_f32("exp10", oracle.linspace_nt2(2, PI, 7))) <= 5
    assert nt2_ulpdist(oracle.logspace_nt2(2, PI, 1, regular=True)[0], oracle.map_f32("exp10", np.float32([PI]))[0]) <= 1
    assert nt2_ulpdist(oracle.logspace_nt2(2, PI, 1)[0], PI) <= 1


def test_mirror_colon_counts_match_oracle(oracle):
    rng = np.random.default_rng(5)
    for _ in range(3000):
        lo, hi = rng.uniform(-50, 50, 2)
        s = rng.choice([rng.uniform(-3, 3), rng.choice([0.1, 0.2, 0.3, 0.7, -0.1, -0.3, 1.0, -1.0])])
        assert E.colon_count(lo, s, hi) == oracle.colon_size_nt2(lo, s, hi), (lo, s, hi)
    assert E.colon(3, 7).args[0].numel == 5 and E.colon(7, 3).args[0].numel == 0
    assert E.linspace(0, 1).args[2].args[0].numel == 100 and E.logspace(0, 1).args[0].args[0].numel == 50


# ------------------------------------------------------------------- GPU --
def _run(dev, expr, n, prec, mode, offset=0, dtype=torch.float32):
    out = torch.full((n,), 7, dtype=dtype, device=dev)
    E.assign([out], [expr], precision=prec, force_generic=mode, offset=offset,
             count=None if offset == 0 else n - offset)
    torch.cuda.synchronize()
    return out.cpu().numpy()


MODES = pytest.mark.parametrize("mode", [1, 2], ids=["compiled", "interpreter"])


@pytest.mark.gpu
@MODES
def test_generative_leaves_bit_exact(dev, oracle, mode):
    cases = [(E.colon(0, 9), oracle.colon_nt2(0, 9)), (E.colon(0, 0.3, 1), oracle.colon_nt2(0, 0.3, 1)),
             (E.colon(-2.5, 0.1, 1e4), oracle.colon_nt2(-2.5, 0.1, 1e4)),
             (E.linspace(-1, 1, 257), oracle.linspace_nt2(-1, 1, 257)),
             (E.linspace(0, 1, 100003), oracle.linspace_nt2(0, 1, 100003)),
             (E.linspace(3, 3, 1), oracle.linspace_nt2(3, 3, 1)),
             (E.logspace(-3, 2, 4099), oracle.logspace_nt2(-3, 2, 4099)),
             (E.logspace(2, PI, 7), oracle.logspace_nt2(2, PI, 7))]
    for e, ref in cases:
        got = _run(dev, e, ref.size, L.PREC_NT2, mode)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), ref.size


@pytest.mark.gpu
@MODES
def test_generative_in_expressions_and_ranges(dev, oracle, mode):
    n = (1 << 25) + 8  # positions past 2^24 round to even floats, as enumerate<float>(p) does
    rng = np.random.default_rng(9)
    x = rng.standard_normal(n).astype(np.float32)
    tx = torch.from_numpy(x).to(dev)
    X = E.Table(tx)
    e = E.sin(E.linspace(0, 1e4, n)) * X + E.colon(1, n) - E.cos(E.colon(0, 1e-3, 2))
    lin, col, c2 = oracle.linspace_nt2(0, 1e4, n), oracle.colon_nt2(1, n), oracle.colon_nt2(0, 1e-3, 2)
    assert lin.size == col.size == n and c2.size == 2001
    with pytest.raises(ValueError):  # 2001 elements do not fit n
        _run(dev, e, n, L.PREC_NT2, mode)
    e = E.sin(E.linspace(0, 1e4, n)) * X + E.colon(1, n)
    ref = oracle.map_f32("sin", lin) * x + col
    got = _run(dev, e, n, L.PREC_NT2, mode)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    # a partial range evaluates the leaf at absolute positions
    off = 1000
    got = _run(dev, E.colon(0, 1, n - 1) * 2.0, n, L.PREC_NT2, mode, offset=off)
    assert (got[:off] == 7).all()
    assert np.array_equal(got[off:], np.arange(off, n, dtype=np.int64).astype(np.float32) * np.float32(2))


@pytest.mark.gpu
@MODES
def test_index_leaf_uint8_wraps(dev, mode):
    n = 1000
    e = E.Node("INDEX", (), L.U8, numel=n) + E.Node("CONST", (), L.U8, imm=3.0)
    got = _run(dev, e, n, L.PREC_NT2, mode, dtype=torch.uint8)
    assert np.array_equal(got, ((np.arange(n) + 3) & 255).astype(np.uint8))


@pytest.mark.gpu
def test_generative_fast_policy_is_correctly_rounded(dev, oracle):
    """Under the fast policy colon/linspace take one fused rounding: the
    value nearest p*s + l."""
    n = E.colon_count(-2.5, 0.1, 1e4)
    got = _run(dev, E.colon(-2.5, 0.1, 1e4), n, L.PREC_FAST, 1)
    p = np.arange(got.size, dtype=np.float64)
    exact = p * np.float64(f(0.1)) + np.float64(f(-2.5))
    assert got.size == oracle.colon_size_nt2(-2.5, 0.1, 1e4)
    assert (np.abs(got - exact) <= 0.5 * np.spacing(np.abs(exact).astype(np.float32)) * 1.0000001).all()


def test_generative_size_mismatch_raises():
    with pytest.raises(ValueError):
        E._check_generative_sizes([E.colon(0, 9)], 11)
    with pytest.raises(ValueError):
        E._check_generative_sizes([E.ones(3) + E.colon(0, 8)], 10)
    E._check_generative_sizes([E.ones(3) + E.colon(0, 8)], 9)
    E._check_generative_sizes([E.zeros(2, 5) * 2.0], 10)
