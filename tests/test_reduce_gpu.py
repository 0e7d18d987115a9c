"""sum / dot on the GPU against the exact superaccumulator oracle and NT2's
known answers.  The kernel accumulates compensated FP32 (TwoSum) and combines
blocks in FP64, so on a well-conditioned input its FP64 result is within a few
ulps of double of the exact sum, far inside FP32's own rounding."""
import numpy as np
import pytest
import torch

from helpers import reduction_ill, reduction_well

pytestmark = pytest.mark.gpu

EPS32 = float(np.finfo(np.float32).eps)


@pytest.fixture(scope="module")
def red(lib, dev):
    return lib.Reducer(dev)


def _run(red, dev, x, y=None):
    tx = torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    ty = None if y is None else torch.from_numpy(np.ascontiguousarray(y)).to(dev)
    o64, o32 = red(tx, ty)
    torch.cuda.synchronize()
    return float(o64.item()), float(o32.item())


def test_known_answers(red, dev):
    assert _run(red, dev, np.ones(133, np.float32)) == (133.0, 133.0)
    a = np.arange(1, 10, dtype=np.float32)
    assert _run(red, dev, a)[0] == 45.0
    a[-1] = 0
    assert _run(red, dev, a)[0] == 36.0
    y = np.array([[i - j for j in range(1, 4)] for i in range(1, 6)], np.float32).ravel()
    assert _run(red, dev, y, y)[0] == 55.0


@pytest.mark.parametrize("n", [0, 1, 3, 5, 17, 1023, 1 << 16])
def test_small_and_ragged(red, dev, oracle, n):
    x, y = reduction_well(max(n, 1), seed=n)
    x, y = x[:n], y[:n]
    assert _run(red, dev, x)[0] == pytest.approx(oracle.exact_sum(x)[0], rel=1e-12, abs=1e-30)
    assert _run(red, dev, x, y)[0] == pytest.approx(oracle.exact_sum(x, y)[0], rel=1e-12, abs=1e-30)


def test_misaligned_input(red, dev, oracle):
    x, y = reduction_well(100001)
    tx, ty = torch.from_numpy(x).to(dev), torch.from_numpy(y).to(dev)
    o64, _ = red(tx[1:], ty[1:])
    torch.cuda.synchronize()
    assert o64.item() == pytest.approx(oracle.exact_sum(x[1:], y[1:])[0], rel=1e-12)


@pytest.mark.parametrize("n", [1 << 24, 1 << 28])
def test_well_conditioned(red, dev, oracle, n):
    x, y = reduction_well(n)
    for yy in (None, y):
        exact, absum = oracle.exact_sum(x, yy)
        got64, got32 = _run(red, dev, x, yy)
        err = abs(got64 - exact)
        print(f"\n{'dot' if yy is not None else 'sum'} n={n}: exact {exact:.17g} got {got64:.17g} "
              f"rel err {err / abs(exact):.3e}; cond {absum / abs(exact):.3g}")
        assert err <= 4 * EPS32 ** 2 * absum + 1e-15 * abs(exact)
        assert got32 == np.float32(got64)
        # deterministic: a second run gives the same bits
        assert _run(red, dev, x, yy)[0] == got64


@pytest.mark.parametrize("n", [1 << 22, 1 << 28])
def test_ill_conditioned(red, dev, oracle, n):
    x = reduction_ill(n)
    exact, absum = oracle.exact_sum(x)
    got64, _ = _run(red, dev, x)
    naive32 = oracle.sum_nt2(x)
    err = abs(got64 - exact)
    print(f"\nill sum n={n}: cond {absum / abs(exact):.3g} exact {exact:.10g} got {got64:.10g} "
          f"rel err {err / abs(exact):.3e}; NT2 fold rel err {abs(naive32 - exact) / abs(exact):.3e}")
    # compensated FP32: error bounded by a small multiple of eps^2 * sum|x|
    assert err <= 64 * EPS32 ** 2 * absum
    assert _run(red, dev, x)[0] == got64


def _noalloc(lib, dev, x, y=None):
    import ctypes
    tx = torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    ty = None if y is None else torch.from_numpy(np.ascontiguousarray(y)).to(dev)
    o64 = torch.zeros(1, dtype=torch.float64, device=dev)
    o32 = torch.zeros(1, dtype=torch.float32, device=dev)
    lib.check(lib.load().nt2g_reduce_f32_noalloc(ctypes.c_void_p(tx.data_ptr()),
                                                  None if ty is None else ctypes.c_void_p(ty.data_ptr()),
                                                  tx.numel(), ctypes.c_void_p(o64.data_ptr()),
                                                  ctypes.c_void_p(o32.data_ptr()), lib._stream()))
    torch.cuda.synchronize()
    return float(o64.item()), float(o32.item())


@pytest.mark.parametrize("n", [1 << 22, 1 << 28])
def test_ill_conditioned_dot(red, lib, dev, oracle, n):
    """dot(x, y) at condition number ~1e10 against the exact dot (FP32
    products are exact in FP64, accumulated exactly), through the workspace
    and the no-allocation entry points.  Compensated dot (TwoProd + TwoSum):
    error within 64 eps^2 sum|x*y|; NT2's naive fold loses every digit."""
    from helpers import reduction_ill_dot
    x, y = reduction_ill_dot(n)
    exact, absum = oracle.exact_sum(x, y)
    cond = absum / abs(exact)
    assert cond > 1e9
    naive = oracle.sum_nt2(x, y)
    for name, fn in (("workspace", lambda: _run(red, dev, x, y)), ("noalloc", lambda: _noalloc(lib, dev, x, y))):
        got64, got32 = fn()
        err = abs(got64 - exact)
        print(f"\nill dot n={n} ({name}): cond {cond:.3g} exact {exact:.10g} got {got64:.10g} "
              f"rel err {err / abs(exact):.3e}; NT2 fold rel err {abs(naive - exact) / abs(exact):.3e}")
        assert err <= 64 * EPS32 ** 2 * absum
        assert got32 == np.float32(got64)
        assert fn()[0] == got64  # deterministic


def test_zero_length_writes_zero(red, lib, dev):
    """n = 0 through both entry points: the outputs, pre-filled with garbage,
    read 0 (the kernel still runs and writes them; the outputs are checked
    reachable even for an empty reduction)."""
    import ctypes
    x = torch.empty(0, device=dev)
    for entry in ("workspace", "noalloc"):
        o64 = torch.full((1,), 123.5, dtype=torch.float64, device=dev)
        o32 = torch.full((1,), -7.0, dtype=torch.float32, device=dev)
        if entry == "workspace":
            ws = torch.empty(red.ws.numel(), dtype=torch.uint8, device=dev)
            lib.check(lib.load().nt2g_reduce_f32(ctypes.c_void_p(x.data_ptr()), None, 0, ctypes.c_void_p(ws.data_ptr()),
                                                 ws.numel(), ctypes.c_void_p(o64.data_ptr()),
                                                 ctypes.c_void_p(o32.data_ptr()), lib._stream()))
        else:
            lib.check(lib.load().nt2g_reduce_f32_noalloc(ctypes.c_void_p(x.data_ptr()), None, 0,
                                                          ctypes.c_void_p(o64.data_ptr()),
                                                          ctypes.c_void_p(o32.data_ptr()), lib._stream()))
        torch.cuda.synchronize()
        assert o64.item() == 0.0 and o32.item() == 0.0, entry
