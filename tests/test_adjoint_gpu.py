"""Fused forward + reverse-mode Black-Scholes kernel against the FP64
analytic vector-Jacobian product and FP64 central finite differences; the
kernel wrapped in a torch.autograd.Function (test harness only)."""
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


def _rel_err(got, ref, floor):
    return np.abs(got.astype(np.float64) - ref) / np.maximum(np.abs(ref), floor)


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
    # floor for near-zero gradients: 1e-4 of the gradient's typical scale
    # (|seed| * the largest partial of its kind over the batch)
    names = ["dS", "dK", "dT", "dsigma", "dr"]
    for name, g, r in zip(names, got[2:], ref):
        floor = 1e-4 * np.quantile(np.abs(r), 0.99)
        e = _rel_err(g, r, floor)
        print(f"\n{name}: max rel err {e.max():.3e} (floor {floor:.3e}), p99.9 {np.quantile(e, 0.999):.3e}")
        assert e.max() <= REL_TOL * 10 and np.quantile(e, 0.999) <= REL_TOL, name
    c64, p64, terms = oracle.blackscholes_f64(S, K, T, R, sig)
    scale = np.maximum(np.abs(terms[:, 0]), np.abs(terms[:, 1]))
    assert (np.abs(got[0] - c64) / np.spacing(scale.astype(np.float32))).max() <= 8


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
    for k in range(5):
        floor = 1e-4 * np.quantile(np.abs(fd[k]), 0.99)
        e = _rel_err(got[k], fd[k], floor)
        assert e.max() <= 1e-4, (k, e.max())


def test_autograd_function_backward(lib, dev, oracle):
    n = 4099
    S, K, T, sig = bs_inputs(n, seed=1004, sigma_table=True)
    ts = [torch.from_numpy(a).to(dev).requires_grad_(True) for a in (S, K, T, sig)]
    c, p = BlackScholesFn.apply(*ts)
    (c.sum() + 2.0 * p.sum()).backward()
    ref = oracle.blackscholes_vjp_f64(S, K, T, sig, R, np.ones(n, np.float32), np.full(n, 2.0, np.float32))
    for tt, r in zip(ts, ref[:4]):
        floor = 1e-4 * np.quantile(np.abs(r), 0.99)
        assert _rel_err(tt.grad.cpu().numpy(), r, floor).max() <= 1e-4
