"""Fused Black-Scholes on the GPU against the oracle.

Parity: the NT2 policy (fused kernel and generic interpreter) is bit-identical
to the CPU restatement of NT2's evaluation on the same seeded inputs.

The fast policy is checked against FP64 with the conditioned metric: the error
in ulps of the larger of the two cancelling terms (call = S N(d1) - K e^-rT
N(d2)), the terms floored at 2^-102 (below that N(d) itself is subnormal in
FP32 and both NT2 and the kernel flush it).  Rounding of d1/d2 is amplified
by |d| times N(d)'s log-derivative (~d^2 in the tail) for any FP32
evaluation, NT2's included.  Stated bound (helpers.BS_FAST_*): max <= 14,
p99.9 <= 6, mean <= 1.1, and <= 8 on the options whose |d1|, |d2| <= 2; the
max is also no worse than NT2's own float evaluation of the same options."""
import numpy as np
import pytest
import torch

from helpers import BS_FAST_CORE, BS_FAST_MAX, BS_FAST_MEAN, BS_FAST_P999, bs_inputs, conditioned_ulp
from nt2_gb300 import expr as E

pytestmark = pytest.mark.gpu

R, SIGMA = 0.02, 0.30


def _dev(dev, *arrs):
    return [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in arrs]


def _run_direct(lib, dev, S, K, T, prec, sig=None):
    tS, tK, tT = _dev(dev, S, K, T)
    tsig = _dev(dev, sig)[0] if sig is not None else None
    c, p = torch.empty_like(tS), torch.empty_like(tS)
    lib.blackscholes(tS, tK, tT, c, p, R, sigma=tsig, sigma_s=SIGMA, precision=prec)
    torch.cuda.synchronize()
    return c.cpu().numpy(), p.cpu().numpy()


def _bits_equal(a, b):
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("n", [1, 3, 5, 4099, 1 << 20])
def test_nt2_policy_bit_exact(lib, dev, oracle, n):
    S, K, T = bs_inputs(n)
    c, p = _run_direct(lib, dev, S, K, T, lib.PREC_NT2)
    rc, rp = oracle.blackscholes(S, K, T, R, SIGMA)
    assert _bits_equal(c, rc) and _bits_equal(p, rp)


def test_nt2_policy_bit_exact_sigma_table(lib, dev, oracle):
    S, K, T, sig = bs_inputs(1 << 18, seed=1004, sigma_table=True)
    c, p = _run_direct(lib, dev, S, K, T, lib.PREC_NT2, sig)
    rc, rp = oracle.blackscholes(S, K, T, R, sig)
    assert _bits_equal(c, rc) and _bits_equal(p, rp)


FLOOR = 2.0 ** -102


def _fast_errors(oracle, S, K, T, c, p, sig=SIGMA):
    c64, p64, terms = oracle.blackscholes_f64(S, K, T, R, sig)
    sc = np.maximum(np.maximum(np.abs(terms[:, 0]), np.abs(terms[:, 1])), FLOOR)
    sp = np.maximum(np.maximum(np.abs(terms[:, 2]), np.abs(terms[:, 3])), FLOOR)
    return conditioned_ulp(c, c64, sc), conditioned_ulp(p, p64, sp)


def _d12(S, K, T, sig):
    s, k, t, v = (np.asarray(a, np.float64) for a in (S, K, T, sig))
    d1 = (np.log(s / k) + (R + 0.5 * v * v) * t) / (v * np.sqrt(t))
    return d1, d1 - v * np.sqrt(t)


def _check_fast(oracle, S, K, T, c, p, sig=SIGMA, label="", fused=True):
    """fused: the fused kernel's stated bound (helpers.BS_FAST_*).  Otherwise
    (the expression evaluated as written, four normcdf calls through the
    compiled kernel or the interpreter): no worse than NT2's own float
    evaluation in mean, p99.9 and max."""
    ec, ep = _fast_errors(oracle, S, K, T, c, p, sig)
    rc, rp = oracle.blackscholes(S, K, T, R, sig)
    nc, np_ = _fast_errors(oracle, S, K, T, rc, rp, sig)
    q = lambda e: np.quantile(e, 0.999)  # noqa: E731
    print(f"\n{label} fast vs FP64 (conditioned ulp): call max {ec.max():.2f} mean {ec.mean():.3f} "
          f"p99.9 {q(ec):.2f}; put max {ep.max():.2f} mean {ep.mean():.3f} p99.9 {q(ep):.2f}")
    print(f"{label} NT2 restatement vs FP64: call max {nc.max():.2f} mean {nc.mean():.3f} p99.9 {q(nc):.2f}; "
          f"put max {np_.max():.2f} mean {np_.mean():.3f} p99.9 {q(np_):.2f}")
    for f, nn in ((ec, nc), (ep, np_)):
        if fused:
            assert f.max() <= BS_FAST_MAX and f.max() <= nn.max()
            assert q(f) <= BS_FAST_P999 and f.mean() <= BS_FAST_MEAN
        else:
            assert f.mean() <= nn.mean() and q(f) <= q(nn) and f.max() <= nn.max()
    d1, d2 = _d12(S, K, T, np.broadcast_to(sig, S.shape))
    core = (np.abs(d1) <= 2) & (np.abs(d2) <= 2)
    print(f"{label} |d|<=2 ({core.mean():.0%} of options): call max {ec[core].max():.2f} put max {ep[core].max():.2f}")
    assert ec[core].max() <= BS_FAST_CORE and ep[core].max() <= BS_FAST_CORE
    return ec, ep


def test_fast_policy_conditioned_error(lib, dev, oracle):
    S, K, T = bs_inputs(1 << 20)
    c, p = _run_direct(lib, dev, S, K, T, lib.PREC_FAST)
    _check_fast(oracle, S, K, T, c, p, label="sigma=0.30")


def test_fast_policy_sigma_table_and_odd_sizes(lib, dev, oracle):
    S, K, T, sig = bs_inputs(1 << 20, seed=1004, sigma_table=True)
    c, p = _run_direct(lib, dev, S, K, T, lib.PREC_FAST, sig)
    _check_fast(oracle, S, K, T, c, p, sig, label="sigma~U[0.05,0.8]")
    big = _run_direct(lib, dev, S, K, T, lib.PREC_FAST, sig)
    for n in (1, 7, 4101):  # odd sizes: same values as the same options in the big batch
        c, p = _run_direct(lib, dev, S[:n], K[:n], T[:n], lib.PREC_FAST, sig[:n])
        assert np.array_equal(c, big[0][:n]) and np.array_equal(p, big[1][:n])


def test_fast_policy_extreme_volatility(lib, dev, oracle):
    """sigma up to 4 (sigma sqrt T up to 12.6): |d1| and |d2| far apart and
    both tails reached; paired (aligned) and single (odd-size) evaluation
    agree bit for bit."""
    rng = np.random.default_rng(1010)
    n = 1 << 18
    S, K, T = bs_inputs(n, seed=1010)
    sig = rng.uniform(1.0, 4.0, n).astype(np.float32)
    c, p = _run_direct(lib, dev, S, K, T, lib.PREC_FAST, sig)
    _check_fast(oracle, S, K, T, c, p, sig, label="sigma~U[1,4]")
    for m in (5, 4097):
        cs, ps = _run_direct(lib, dev, S[:m], K[:m], T[:m], lib.PREC_FAST, sig[:m])
        assert np.array_equal(cs, c[:m]) and np.array_equal(ps, p[:m])


def test_misaligned_tables_take_the_scalar_path(lib, dev, oracle):
    n = 1001
    S, K, T = bs_inputs(n + 1)
    tS, tK, tT = _dev(dev, S, K, T)
    c, p = torch.empty_like(tS), torch.empty_like(tS)
    # views starting one float in: not 16-byte aligned
    lib.blackscholes(tS[1:], tK[1:], tT[1:], c[1:], p[1:], R, sigma_s=SIGMA, precision=lib.PREC_NT2)
    torch.cuda.synchronize()
    rc, rp = oracle.blackscholes(S[1:], K[1:], T[1:], R, SIGMA)
    assert _bits_equal(c.cpu().numpy()[1:], rc) and _bits_equal(p.cpu().numpy()[1:], rp)
    # fast policy: the one-option-at-a-time path equals the paired path bit for bit
    sig = np.random.default_rng(7).uniform(0.05, 4.0, n + 1).astype(np.float32)
    tsig = _dev(dev, sig)[0]
    for sigma, sig_s in ((None, SIGMA), (tsig, 0.0)):
        c.zero_(), p.zero_()
        lib.blackscholes(tS[1:], tK[1:], tT[1:], c[1:], p[1:], R, sigma=None if sigma is None else sigma[1:],
                         sigma_s=sig_s, precision=lib.PREC_FAST)
        ca, pa = _run_direct(lib, dev, S[1:], K[1:], T[1:], lib.PREC_FAST, None if sigma is None else sig[1:])
        torch.cuda.synchronize()
        assert _bits_equal(c.cpu().numpy()[1:], ca) and _bits_equal(p.cpu().numpy()[1:], pa)


def bs_expr(S, K, T, sig, r):
    sq = E.sqrt(T)
    d1 = (E.log(S / K) + E.fma(E.sqr(sig), 0.5, r) * T) / (sig * sq)
    d2 = E.fnms(sig, sq, d1)
    e = K * E.exp(-r * T)
    return E.fnms(e, E.normcdf(d2), S * E.normcdf(d1)), E.fnms(S, E.normcdf(-d1), e * E.normcdf(-d2))


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
def test_expression_path_binds_the_fused_kernel(lib, dev, oracle, prec):
    n = 1 << 16
    S, K, T = bs_inputs(n)
    tS, tK, tT = _dev(dev, S, K, T)
    c, p = torch.empty_like(tS), torch.empty_like(tS)
    prog = E.assign([c, p], bs_expr(E.Table(tS), E.Table(tK), E.Table(tT), SIGMA, R), precision=prec)
    assert prog.info().kernel_name == b"blackscholes"
    dc, dp = _run_direct(lib, dev, S, K, T, prec)
    torch.cuda.synchronize()
    assert _bits_equal(c.cpu().numpy(), dc) and _bits_equal(p.cpu().numpy(), dp)


def test_generic_interpreter_reproduces_nt2(lib, dev, oracle):
    n = 50001
    S, K, T = bs_inputs(n)
    tS, tK, tT = _dev(dev, S, K, T)
    c, p = torch.empty_like(tS), torch.empty_like(tS)
    E.assign([c, p], bs_expr(E.Table(tS), E.Table(tK), E.Table(tT), E.Scalar(SIGMA), E.Scalar(R)),
             precision=lib.PREC_NT2, force_generic=True)
    torch.cuda.synchronize()
    rc, rp = oracle.blackscholes(S, K, T, R, SIGMA)
    assert _bits_equal(c.cpu().numpy(), rc) and _bits_equal(p.cpu().numpy(), rp)
    # the interpreter's fast policy evaluates the same graph with FMAs
    E.assign([c, p], bs_expr(E.Table(tS), E.Table(tK), E.Table(tT), SIGMA, R), precision=lib.PREC_FAST,
             force_generic=True)
    torch.cuda.synchronize()
    _check_fast(oracle, S, K, T, c.cpu().numpy(), p.cpu().numpy(), label="interpreter", fused=False)


def test_partial_transform_range(lib, dev, oracle):
    n = 21
    S, K, T = bs_inputs(n)
    tS, tK, tT = _dev(dev, S, K, T)
    c, p = torch.zeros_like(tS), torch.zeros_like(tS)
    E.assign([c, p], bs_expr(E.Table(tS), E.Table(tK), E.Table(tT), SIGMA, R), precision=lib.PREC_NT2,
             offset=6, count=6)
    torch.cuda.synchronize()
    rc, _ = oracle.blackscholes(S, K, T, R, SIGMA)
    got = c.cpu().numpy()
    assert (got[:6] == 0).all() and (got[12:] == 0).all()
    assert _bits_equal(got[6:12], rc[6:12])


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
def test_demo_form(lib, dev, oracle, prec):
    n = 1 << 16
    S, X, T = bs_inputs(n)
    rng = np.random.default_rng(3)
    rt = rng.uniform(0.01, 0.05, n).astype(np.float32)
    vt = rng.uniform(0.1, 0.5, n).astype(np.float32)
    tS, tX, tT, trt, tvt = _dev(dev, S, X, T, rt, vt)
    R_ = torch.empty_like(tS)
    lib.blackscholes_demo(tS, tX, tT, R_, r_t=trt, v_t=tvt, precision=prec)
    torch.cuda.synchronize()
    ref = oracle.blackscholes_demo(S, X, T, rt, vt)
    got = R_.cpu().numpy()
    if prec == lib.PREC_NT2:
        assert _bits_equal(got, ref)
    else:
        scale = np.maximum(np.abs(S), np.abs(X)).astype(np.float32)
        assert (np.abs(got.astype(np.float64) - ref) / np.spacing(scale)).max() <= 8
    # through the expression front end, with scalar r and v: binds the demo kernel
    v, r = 0.3, 0.02
    Sx, Xx, Tx = E.Table(tS), E.Table(tX), E.Table(tT)
    da = E.sqrt(Tx)
    d1 = E.log(Sx / Xx) + (E.fma(E.sqr(E.Scalar(v)), 0.5, r) * Tx) / (E.Scalar(v) * da)
    out = torch.empty_like(tS)
    prog = E.assign([out], [E.fnms(Xx * E.exp(-r * Tx), E.fastnormcdf(E.fnms(v, da, d1)), Sx * E.fastnormcdf(d1))],
                    precision=prec)
    assert prog.info().kernel_name == b"generic"  # v is a scalar slot in one place and a constant in another
    vs = E.Scalar(v)
    d1 = E.log(Sx / Xx) + (E.fma(E.sqr(vs), 0.5, r) * Tx) / (vs * da)
    prog = E.assign([out], [E.fnms(Xx * E.exp(-r * Tx), E.fastnormcdf(E.fnms(vs, da, d1)), Sx * E.fastnormcdf(d1))],
                    precision=prec)
    assert prog.info().kernel_name == b"blackscholes_demo"
    torch.cuda.synchronize()
    ref = oracle.blackscholes_demo(S, X, T, r, v)
    got = out.cpu().numpy()
    if prec == lib.PREC_NT2:
        assert _bits_equal(got, ref)


@pytest.mark.parametrize("sigma_table", [False, True], ids=["sigma_scalar", "sigma_table"])
def test_pipelined_kernel_tile_boundaries(lib, dev, oracle, sigma_table):
    """The bulk-copy pipelined kernel (aligned tables of 2^22 options or more:
    persistent blocks over tiles of 1024 options, the part past the last whole
    tile priced with plain loads) at sizes around its tile boundaries and
    either side of its threshold: NT2 policy bit-identical to the oracle, and
    no bounded wait ever gave up."""
    import ctypes
    from helpers import bs_inputs
    for n in (1025, (1 << 22) - 1, 1 << 22, (1 << 22) + 1023, (1 << 22) + 1024 * 777 + 3):
        ins = bs_inputs(n, seed=n, sigma_table=sigma_table)
        t = [torch.from_numpy(a).to(dev) for a in ins]
        c, p = torch.empty_like(t[0]), torch.empty_like(t[0])
        if sigma_table:
            lib.blackscholes(t[0], t[1], t[2], c, p, 0.02, sigma=t[3], precision=lib.PREC_NT2)
            rc, rp = oracle.blackscholes(ins[0], ins[1], ins[2], 0.02, ins[3])
        else:
            lib.blackscholes(t[0], t[1], t[2], c, p, 0.02, sigma_s=0.3, precision=lib.PREC_NT2)
            rc, rp = oracle.blackscholes(ins[0], ins[1], ins[2], 0.02, 0.3)
        torch.cuda.synchronize()
        assert np.array_equal(c.cpu().numpy().view(np.uint32), rc.view(np.uint32)), n
        assert np.array_equal(p.cpu().numpy().view(np.uint32), rp.view(np.uint32)), n
    count = ctypes.c_uint64()
    lib.check(lib.load().nt2g_wait_timeouts(ctypes.byref(count)))
    assert count.value == 0
