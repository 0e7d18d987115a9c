"""Fused forward + reverse-mode Black-Scholes kernel against the FP64
analytic vector-Jacobian product and FP64 central finite differences; the
kernel wrapped in a torch.autograd.Function (test harness only).

Relative gradient error is measured against each gradient's term scale -- the
sum of the magnitudes of the terms its analytic formula adds (for dS:
|gc N(d1)| + |gp N(-d1)|) -- which is the gradient's own magnitude except
where the seeds make it cancel toward zero.  Stated floor for near-zero
Greeks: 1e-10 of the Greek's natural scale, (|gc|+|gp|) times 1 (delta, dK),
S (theta), S*sqrt(T) (vega), K*T (rho).  Below it a Greek is zero for any
practical purpose and FP32's rounding of d1, amplified by d1^2 in phi(d1)
(|d1| > 8), dominates.  Tolerance 1e-5."""
import numpy as np
import pytest
import torch

from helpers import bs_inputs

pytestmark = pytest.mark.gpu

R = 0.02
REL_TOL = 1e-5


class BlackScholesFn(torch.autograd.Function):
    """call, put = BS(S, K, T, sigma); backward through nt2g_blackscholes_vjp_f32.
    Forward runs the same fused kernel with zero seeds (it writes call/put)."""

    @staticmethod
    def forward(ctx, S, K, T, sigma):
        from nt2_gb300 import lib
        outs = [torch.empty_like(S) for _ in range(7)]
        z = torch.zeros_like(S)
        lib.blackscholes_vjp(S, K, T, sigma, R, z, z, outs)
        ctx.save_for_backward(S, K, T, sigma)
        return outs[0], outs[1]

    @staticmethod
    def backward(ctx, gc, gp):
        from nt2_gb300 import lib
        S, K, T, sigma = ctx.saved_tensors
        outs = [torch.empty_like(S) for _ in range(7)]
        lib.blackscholes_vjp(S, K, T, sigma, R, gc.contiguous(), gp.contiguous(), outs)
        return outs[2], outs[3], outs[4], outs[5]


SCALE_FLOOR = 2.0 ** -100  # below this FP32 holds a gradient's terms only as subnormals


def _natural_floor(S, K, T, gc, gp):
    g = np.abs(gc.astype(np.float64)) + np.abs(gp.astype(np.float64))
    s, k, t = (a.astype(np.float64) for a in (S, K, T))
    return [1e-10 * g * x for x in (np.ones_like(s), np.ones_like(s), s, s * np.sqrt(t), k * t)]


def _scaled_err(got, ref, scale, floor=0.0):
    """|got - ref| / max(term scale, natural floor, 2^-100)."""
    err = np.abs(np.asarray(got, np.float64) - ref)
    return err / np.maximum(np.maximum(scale, floor), SCALE_FLOOR)


def test_vjp_against_fp64_analytic(lib, dev, oracle):
    n = 1 << 20
    S, K, T, sig = bs_inputs(n, seed=1004, sigma_table=True)
    rng = np.random.default_rng(1005)
    gc, gp = rng.uniform(-1, 1, n).astype(np.float32), rng.uniform(-1, 1, n).astype(np.float32)
    t = [torch.from_numpy(a).to(dev) for a in (S, K, T, sig, gc, gp)]
    outs = [torch.empty_like(t[0]) for _ in range(7)]
    lib.blackscholes_vjp(t[0], t[1], t[2], t[3], R, t[4], t[5], outs)
    torch.cuda.synchronize()
    got = [o.cpu().numpy() for o in outs]
    ref = oracle.blackscholes_vjp_f64(S, K, T, sig, R, gc, gp)
    scale = oracle.blackscholes_vjp_scale_f64(S, K, T, sig, R, gc, gp)
    floors = _natural_floor(S, K, T, gc, gp)
    names = ["dS", "dK", "dT", "dsigma", "dr"]
    for name, g, r, sc, fl in zip(names, got[2:], ref, scale, floors):
        e = _scaled_err(g, r, sc, fl)
        plain = np.abs(g.astype(np.float64) - r) / np.where(r != 0, np.abs(r), 1.0)
        print(f"\n{name}: max rel err (term scale) {e.max():.3e} mean {e.mean():.3e}; "
              f"plain rel err median {np.median(plain):.3e}")
        assert e.max() <= REL_TOL, name
    # the forward half is the fast forward kernel, bit for bit
    fc, fp = torch.empty_like(t[0]), torch.empty_like(t[0])
    lib.blackscholes(t[0], t[1], t[2], fc, fp, R, sigma=t[3])
    torch.cuda.synchronize()
    assert np.array_equal(fc.cpu().numpy().view(np.uint32), got[0].view(np.uint32))
    assert np.array_equal(fp.cpu().numpy().view(np.uint32), got[1].view(np.uint32))


PLAIN_FLOOR = 0.1  # of each gradient's RMS over the batch
NAMES = ["dS", "dK", "dT", "dsigma", "dr"]


def _plain_check(label, got, ref):
    """Plain relative error |got - ref| / |ref| <= 1e-5 for every gradient at
    least the floor (a tenth of that gradient's RMS over the batch); below it,
    absolute error <= 1e-5 x floor.  A FP32 gradient that cancels toward zero
    (seeds of opposite sign, or put theta crossing zero) carries an absolute
    error of a few ulps of its terms, so no FP32 evaluation has a relative
    error there."""
    bad = []
    for name, g, r in zip(NAMES, got, ref):
        floor = PLAIN_FLOOR * float(np.sqrt(np.mean(r * r)))
        a = np.abs(r)
        err = np.abs(g.astype(np.float64) - r)
        big = a >= floor
        rel = err[big] / a[big]
        below = err[~big].max() / floor if (~big).any() else 0.0
        print(f"\n{label} {name}: floor {floor:.3e} ({(~big).mean():.2%} of options below); plain rel err max "
              f"{rel.max():.3e} p99.99 {np.quantile(rel, 0.9999):.3e} median {np.median(rel):.3e}; "
              f"below the floor max |err| / floor {below:.3e}")
        if rel.max() > REL_TOL or below > REL_TOL:
            bad.append((label, name, float(rel.max()), float(below)))
    return bad


def test_vjp_plain_relative_error_2e26(lib, dev, oracle):
    """The adjoint workload itself: N = 2^26 options (S~U[5,30], K~U[1,100],
    T~U[0.25,10], sigma~U[0.05,0.8] per option, r = 0.02), seeds gc, gp ~
    U[-1,1], against the FP64 analytic VJP:
      - plain relative error <= 1e-5 above one floor per gradient (a tenth of
        its RMS over the batch), absolute error <= 1e-5 x floor below it;
      - relative error <= 1e-5 against each gradient's term scale everywhere;
      - the pure Greeks of the first 2^24 options (seeds (1, 0) and (0, 1):
        call and put delta, dK, theta, vega, rho), plain relative error as above;
      - a 4096-option sample against FP64 central differences (h = 1e-4
        relative), plain relative error as above."""
    n = 1 << 26
    S, K, T, sig = bs_inputs(n, seed=1004, sigma_table=True)
    rng = np.random.default_rng(1005)
    gc, gp = rng.uniform(-1, 1, n).astype(np.float32), rng.uniform(-1, 1, n).astype(np.float32)
    t = [torch.from_numpy(a).to(dev) for a in (S, K, T, sig, gc, gp)]
    outs = [torch.empty_like(t[0]) for _ in range(7)]
    lib.blackscholes_vjp(t[0], t[1], t[2], t[3], R, t[4], t[5], outs)
    torch.cuda.synchronize()
    got = [o.cpu().numpy() for o in outs[2:]]
    ref = oracle.blackscholes_vjp_f64(S, K, T, sig, R, gc, gp)
    bad = _plain_check("seeds U[-1,1]", got, ref)
    scale = oracle.blackscholes_vjp_scale_f64(S, K, T, sig, R, gc, gp)
    for name, g, r, sc, fl in zip(NAMES, got, ref, scale, _natural_floor(S, K, T, gc, gp)):
        e = _scaled_err(g, r, sc, fl)
        print(f"{name}: term-scale rel err max {e.max():.3e}")
        if e.max() > REL_TOL:
            bad.append(("term scale", name, float(e.max())))
    del scale
    # pure Greeks on the first 2^24 options
    m = 1 << 24
    for seeds, label in (((1.0, 0.0), "call Greeks"), ((0.0, 1.0), "put Greeks")):
        a = np.full(m, seeds[0], np.float32)
        b = np.full(m, seeds[1], np.float32)
        ta, tb = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
        o = [torch.empty(m, device=dev) for _ in range(7)]
        lib.blackscholes_vjp(t[0][:m], t[1][:m], t[2][:m], t[3][:m], R, ta, tb, o)
        torch.cuda.synchronize()
        bad += _plain_check(label, [x.cpu().numpy() for x in o[2:]],
                            oracle.blackscholes_vjp_f64(S[:m], K[:m], T[:m], sig[:m], R, a, b))
    del t, outs
    # central differences on a seeded sample of the batch
    idx = np.random.default_rng(1006).choice(n, 4096, replace=False)
    fd = np.zeros((5, idx.size))
    for j, i in enumerate(idx):
        p = [float(S[i]), float(K[i]), float(T[i]), float(sig[i]), R]
        for k in range(5):
            h = 1e-4 * abs(p[k])
            up, dn = list(p), list(p)
            up[k] += h
            dn[k] -= h
            cu, pu = oracle.blackscholes_point_f64(*up)
            cd, pd = oracle.blackscholes_point_f64(*dn)
            fd[k, j] = (float(gc[i]) * (cu - cd) + float(gp[i]) * (pu - pd)) / (2 * h)
    for k, name in enumerate(NAMES):
        floor = PLAIN_FLOOR * float(np.sqrt(np.mean(ref[k] * ref[k])))
        e = np.abs(got[k][idx].astype(np.float64) - fd[k]) / np.maximum(np.abs(fd[k]), floor)
        print(f"{name}: vs central differences, plain rel err max {e.max():.3e}")
        if e.max() > REL_TOL:
            bad.append(("central differences", name, float(e.max())))
    assert not bad, bad


def test_vjp_against_central_differences(lib, dev, oracle):
    n = 256
    S, K, T, sig = bs_inputs(n, seed=77, sigma_table=True)
    gc = np.ones(n, np.float32)
    gp = np.full(n, 0.5, np.float32)
    t = [torch.from_numpy(a).to(dev) for a in (S, K, T, sig, gc, gp)]
    outs = [torch.empty_like(t[0]) for _ in range(7)]
    lib.blackscholes_vjp(t[0], t[1], t[2], t[3], R, t[4], t[5], outs)
    torch.cuda.synchronize()
    got = [o.cpu().numpy() for o in outs[2:]]
    fd = np.zeros((5, n))
    for i in range(n):
        p = [float(S[i]), float(K[i]), float(T[i]), float(sig[i]), R]
        for k in range(5):
            h = 1e-4 * abs(p[k])
            up, dn = list(p), list(p)
            up[k] += h
            dn[k] -= h
            cu, pu = oracle.blackscholes_point_f64(*up)
            cd, pd = oracle.blackscholes_point_f64(*dn)
            fd[k, i] = (gc[i] * (cu - cd) + gp[i] * (pu - pd)) / (2 * h)
    scale = oracle.blackscholes_vjp_scale_f64(S, K, T, sig, R, gc, gp)
    for k in range(5):
        # central differences carry O(h^2) truncation and ~1e-14/h of FP64
        # cancellation noise (1e-9 absolute for h = 1e-4 * 0.05): floor 1e-4
        e = np.abs(got[k].astype(np.float64) - fd[k]) / np.maximum(scale[k], 1e-4)
        assert e.max() <= 1e-5, (k, e.max())


def test_autograd_function_backward(lib, dev, oracle):
    n = 4099
    S, K, T, sig = bs_inputs(n, seed=1004, sigma_table=True)
    ts = [torch.from_numpy(a).to(dev).requires_grad_(True) for a in (S, K, T, sig)]
    c, p = BlackScholesFn.apply(*ts)
    (c.sum() + 2.0 * p.sum()).backward()
    gc, gp = np.ones(n, np.float32), np.full(n, 2.0, np.float32)
    ref = oracle.blackscholes_vjp_f64(S, K, T, sig, R, gc, gp)
    scale = oracle.blackscholes_vjp_scale_f64(S, K, T, sig, R, gc, gp)
    floors = _natural_floor(S, K, T, gc, gp)
    for tt, r, sc, fl in zip(ts, ref[:4], scale[:4], floors[:4]):
        assert _scaled_err(tt.grad.cpu().numpy(), r, sc, fl).max() <= REL_TOL
