"""Host tables evaluated in place.

Every entry point takes host pointers where the device can reach the memory
(pinned host memory anywhere; any host memory where the device has pageable
memory access, as on Grace-Blackwell).  The kernels then read and write the
host tables over the host link, and the results are bit-identical to the same
call on device tables.  NT2's own CUDA path stages every host table through a
device buffer (modules/arch/cuda/include/nt2/memory/functions/cuda/copy.hpp:24-100).
"""
import ctypes

import numpy as np
import pytest
import torch

from helpers import bs_inputs
from nt2_gb300 import expr as E

pytestmark = pytest.mark.gpu

R, SIGMA = 0.02, 0.30


def _pageable(lib):
    v = ctypes.c_int32(-1)
    lib.check(lib.load().nt2g_host_access(ctypes.byref(v)))
    assert v.value in (0, 1)
    return v.value == 1


def _host(a, kind):
    t = torch.from_numpy(np.ascontiguousarray(a).copy())
    return t.pin_memory() if kind == "pinned" else t


def _bits(t):
    return t.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("kind", ["pageable", "pinned"])
@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
def test_blackscholes_host_tables_in_place(lib, dev, oracle, kind, prec):
    n = 100003
    S, K, T = bs_inputs(n, seed=77)
    hS, hK, hT = (_host(a, kind) for a in (S, K, T))
    hc, hp = _host(np.zeros(n, np.float32), kind), _host(np.zeros(n, np.float32), kind)
    if kind == "pageable" and not _pageable(lib):
        with pytest.raises(lib.Nt2gError):
            lib.blackscholes(hS, hK, hT, hc, hp, R, sigma_s=SIGMA, precision=prec)
        return
    lib.blackscholes(hS, hK, hT, hc, hp, R, sigma_s=SIGMA, precision=prec)
    dS, dK, dT = (t.to(dev) for t in (hS, hK, hT))
    dc, dp = torch.empty_like(dS), torch.empty_like(dS)
    lib.blackscholes(dS, dK, dT, dc, dp, R, sigma_s=SIGMA, precision=prec)
    torch.cuda.synchronize()
    assert np.array_equal(_bits(hc), _bits(dc)) and np.array_equal(_bits(hp), _bits(dp))
    if prec == lib.PREC_NT2:
        rc, rp = oracle.blackscholes(S, K, T, R, SIGMA)
        assert np.array_equal(hc.numpy().view(np.uint32), rc.view(np.uint32))


def test_generic_program_and_reduction_on_host_tables(lib, dev):
    if not _pageable(lib):
        pytest.skip("device has no pageable memory access")
    n = 65537
    rng = np.random.default_rng(78)
    x, y = rng.standard_normal(n).astype(np.float32), rng.uniform(0.5, 2, n).astype(np.float32)
    hx, hy, ho = torch.from_numpy(x), torch.from_numpy(y), torch.zeros(n)
    e = lambda X, Y: E.if_else(X < Y, E.exp(X) * Y, E.log1p(E.abs_(X)) - Y)  # noqa: E731
    for mode in (1, 2):  # compiled kernel, interpreter
        E.assign([ho], [e(E.Table(hx), E.Table(hy))], force_generic=mode)
        dx, dy = hx.to(dev), hy.to(dev)
        do = torch.empty_like(dx)
        E.assign([do], [e(E.Table(dx), E.Table(dy))], force_generic=mode)
        torch.cuda.synchronize()
        assert np.array_equal(_bits(ho), _bits(do)), mode
    # dot on host vectors equals dot on device vectors (same partial order)
    red = lib.Reducer(dev)
    h = [t.item() for t in red(hx, hy)]
    d = [t.item() for t in red(hx.to(dev), hy.to(dev))]
    assert h == d


def test_sigmadelta_in_place_on_host_frames(lib, dev, oracle):
    if not _pageable(lib):
        pytest.skip("device has no pageable memory access")
    from helpers import sigmadelta_frames
    frames = sigmadelta_frames(h=72, w=129, frames=6, seed=79)
    F, H, W = frames.shape
    n = H * W
    rb, rv = frames[0].ravel().copy(), np.ones(n, np.uint8)
    hb, hv = torch.from_numpy(rb.copy()), torch.from_numpy(rv.copy())
    hl = torch.zeros(n, dtype=torch.uint8)
    for k in range(1, F):
        hf = torch.from_numpy(frames[k].ravel().copy())
        lib.sigmadelta(hf, hb, hv, hl)
        torch.cuda.synchronize()
        rb, rv, rl = oracle.sigmadelta(frames[k].ravel(), rb, rv)
        assert np.array_equal(hb.numpy(), rb) and np.array_equal(hv.numpy(), rv) and np.array_equal(hl.numpy(), rl), k
