"""saxpy, expr3, rgb2yuv, sigma-delta and the generic interpreter on the GPU
against the oracle (bit-exact where NT2's arithmetic is reproduced)."""
import numpy as np
import pytest
import torch

from helpers import conditioned_ulp, rgb_planes, sigmadelta_frames, std_ulp
from nt2_gb300 import expr as E

pytestmark = pytest.mark.gpu


def _t(dev, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _eq(a, b):
    return np.array_equal(np.asarray(a).view(np.uint8), np.asarray(b).view(np.uint8))


@pytest.mark.parametrize("n", [0, 1, 5, 1 << 20])
def test_saxpy_bit_exact(lib, dev, oracle, n):
    rng = np.random.default_rng(1003)
    x, y = rng.standard_normal(n).astype(np.float32), rng.standard_normal(n).astype(np.float32)
    a = np.float32(rng.uniform(-2, 2))
    tx, ty = _t(dev, x), _t(dev, y)
    lib.saxpy(float(a), tx, ty)
    ref = oracle.saxpy(a, x, y)
    assert _eq(ty.cpu().numpy(), ref)
    # expression path, in place: Y = alpha*X + Y binds the saxpy kernel
    ty2 = _t(dev, y)
    prog = E.assign([ty2], [float(a) * E.Table(tx) + E.Table(ty2)])
    assert prog.info().kernel_name == b"saxpy"
    torch.cuda.synchronize()
    assert _eq(ty2.cpu().numpy(), ref)


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
def test_expr3(lib, dev, oracle, prec):
    n = (1 << 20) + 3
    rng = np.random.default_rng(1003)
    x, y, z = (rng.standard_normal(n).astype(np.float32) for _ in range(3))
    tx, ty, tz = _t(dev, x), _t(dev, y), _t(dev, z)
    out = torch.empty_like(tx)
    lib.expr3(tx, ty, tz, out, precision=prec)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    if prec == lib.PREC_NT2:
        assert _eq(got, oracle.expr3(x, y, z))
    else:
        e = std_ulp(got, oracle.expr3_f64(x, y, z))
        print(f"\nexpr3 fast vs FP64: max {e.max():.2f} mean {e.mean():.3f} ulp")
        assert e.max() <= 4.0
    out2 = torch.empty_like(tx)
    X, Y, Z = E.Table(tx), E.Table(ty), E.Table(tz)
    prog = E.assign([out2], [E.exp(-E.sqr(X)) * E.sqrt(E.abs_(Y)) + E.log1p(E.abs_(Z))], precision=prec)
    assert prog.info().kernel_name == b"expr3"
    torch.cuda.synchronize()
    assert _eq(out2.cpu().numpy(), got)


def test_rgb2yuv_nt2_policy_bit_exact(lib, dev, oracle):
    n = 1920 * 1080
    r, g, b = rgb_planes(n)
    tr, tg, tb = _t(dev, r), _t(dev, g), _t(dev, b)
    y, u, v = (torch.empty_like(tr) for _ in range(3))
    lib.rgb2yuv(tr, tg, tb, y, u, v, precision=lib.PREC_NT2)
    torch.cuda.synchronize()
    ry, ru, rv = oracle.rgb2yuv(r, g, b)
    assert _eq(y.cpu().numpy(), ry) and _eq(u.cpu().numpy(), ru) and _eq(v.cpu().numpy(), rv)
    # expression path (tie: u, v read the y just stored) binds the same kernel
    y2, u2, v2 = (torch.empty_like(tr) for _ in range(3))
    R, G, B, Y2 = E.Table(tr), E.Table(tg), E.Table(tb), E.Table(y2)
    prog = E.assign([y2, u2, v2], [0.299 * R + 0.587 * G + 0.114 * B, 0.492 * (B - Y2), 0.877 * (R - Y2)],
                    precision=lib.PREC_NT2)
    assert prog.info().kernel_name == b"rgb2yuv"
    torch.cuda.synchronize()
    assert _eq(y2.cpu().numpy(), ry) and _eq(u2.cpu().numpy(), ru) and _eq(v2.cpu().numpy(), rv)


def test_rgb2yuv_accuracy(lib, dev, oracle):
    """Against an extended-precision reference with the same float constants.
    NT2's unfused y is within 2 ulp; its u = 0.492(b - y) inherits y's
    rounding through the b - y cancellation.  The fast policy carries y as a
    double-float: y, u, v within 2 ulp of their own value wherever the
    cancellation leaves at least 2^-20 of the operands, and within one ulp of
    the operands' scale everywhere."""
    n = 1920 * 1080
    r, g, b = rgb_planes(n)
    tr, tg, tb = _t(dev, r), _t(dev, g), _t(dev, b)
    y, u, v = (torch.empty_like(tr) for _ in range(3))
    lib.rgb2yuv(tr, tg, tb, y, u, v, precision=lib.PREC_FAST)
    torch.cuda.synchronize()
    L = np.longdouble
    rl, gl, bl = (a.astype(L) for a in (r, g, b))
    c = [L(np.float32(k)) for k in (0.299, 0.587, 0.114, 0.492, 0.877)]
    yl = c[0] * rl + c[1] * gl + c[2] * bl
    refs = [yl, c[3] * (bl - yl), c[4] * (rl - yl)]
    scales = [yl, c[3] * np.maximum(bl, yl), c[4] * np.maximum(rl, yl)]
    ry, ru, rv = oracle.rgb2yuv(r, g, b)
    assert std_ulp(ry, yl.astype(np.float64)).max() <= 2.0
    print(f"\nNT2 u vs exact: conditioned {conditioned_ulp(ru, refs[1].astype(np.float64), scales[1].astype(np.float64)).max():.2f}")
    for name, got, ref, sc in zip("yuv", (y, u, v), refs, scales):
        got = got.cpu().numpy()
        ref64, sc64 = ref.astype(np.float64), sc.astype(np.float64)
        cond = conditioned_ulp(got, ref64, sc64)
        mild = np.abs(ref64) >= 2.0 ** -20 * np.abs(sc64)
        e = std_ulp(got[mild], ref64[mild])
        print(f"fast {name}: max {e.max():.2f} ulp (mild cancellation), conditioned max {cond.max():.2f}")
        assert e.max() <= 1.0 and cond.max() <= 1.0, name


def _sd_exprs(fr, bkg, var):
    nb = E.selinc(bkg < fr, E.seldec(bkg > fr, bkg))
    d = E.max_(bkg, fr) - E.min_(bkg, fr)  # reads the bkg just stored (tie)
    m = E.adds(E.adds(d, d), d)
    nv = E.if_else(d.ne(0), E.selinc(var < m, E.seldec(var > m, var)), var)
    return nb, nv, E.if_zero_else_one(d < var, 1)


def test_sigmadelta_bit_exact_every_frame(lib, dev, oracle):
    frames = sigmadelta_frames()
    F, H, W = frames.shape
    n = H * W
    bkg0 = frames[0].ravel().copy()
    var0 = np.ones(n, np.uint8)
    tf = _t(dev, frames.reshape(F, n))
    # 1. per-frame kernel   2. expression path (pattern-bound)   3. interpreter
    tb = [_t(dev, bkg0) for _ in range(3)]
    tv = [_t(dev, var0) for _ in range(3)]
    tl = [torch.zeros(n, dtype=torch.uint8, device=dev) for _ in range(3)]
    rb, rv = bkg0.copy(), var0.copy()
    for k in range(1, F):
        rb, rv, rl = oracle.sigmadelta(frames[k].ravel(), rb, rv)
        lib.sigmadelta(tf[k], tb[0], tv[0], tl[0])
        if k < 6:
            prog = E.assign([tb[1], tv[1], tl[1]], _sd_exprs(E.Table(tf[k]), E.Table(tb[1]), E.Table(tv[1])))
            assert prog.info().kernel_name == b"sigmadelta"
            E.assign([tb[2], tv[2], tl[2]], _sd_exprs(E.Table(tf[k]), E.Table(tb[2]), E.Table(tv[2])),
                     force_generic=True)
        torch.cuda.synchronize()
        assert _eq(tb[0].cpu().numpy(), rb) and _eq(tv[0].cpu().numpy(), rv) and _eq(tl[0].cpu().numpy(), rl), k
        if k < 6:
            for j in (1, 2):
                assert _eq(tb[j].cpu().numpy(), rb) and _eq(tv[j].cpu().numpy(), rv), (k, j)
                assert _eq(tl[j].cpu().numpy(), rl), (k, j)


def test_sigmadelta_temporal_fusion(lib, dev, oracle):
    frames = sigmadelta_frames(h=270, w=480, frames=17, seed=9)
    F, H, W = frames.shape
    n = H * W
    rb, rv = frames[0].ravel().copy(), np.ones(n, np.uint8)
    tb, tv = _t(dev, rb), _t(dev, rv)
    tl = torch.zeros((F - 1, n), dtype=torch.uint8, device=dev)
    lib.sigmadelta_frames(_t(dev, frames[1:].reshape(F - 1, n)), tb, tv, tl)
    torch.cuda.synchronize()
    labels = tl.cpu().numpy()
    for k in range(1, F):
        rb, rv, rl = oracle.sigmadelta(frames[k].ravel(), rb, rv)
        assert _eq(labels[k - 1], rl), k
    assert _eq(tb.cpu().numpy(), rb) and _eq(tv.cpu().numpy(), rv)


def test_sigmadelta_exhaustive_byte_triples(lib, dev, oracle):
    """Every (frame, bkg, var) byte triple, 2^24 pixels: the per-frame kernel
    (16-pixel vectors), the fused kernel on one frame (16-pixel and 4-pixel
    paths) and the single-pixel path all equal the CPU restatement."""
    i = np.arange(1 << 24, dtype=np.uint32)
    f, b, v = (i & 255).astype(np.uint8), ((i >> 8) & 255).astype(np.uint8), (i >> 16).astype(np.uint8)
    rb, rv, rl = oracle.sigmadelta(f, b, v)
    tf = _t(dev, f)
    # per-frame kernel
    tb, tv, tl = _t(dev, b), _t(dev, v), torch.empty_like(tf)
    lib.sigmadelta(tf, tb, tv, tl)
    torch.cuda.synchronize()
    assert _eq(tb.cpu().numpy(), rb) and _eq(tv.cpu().numpy(), rv) and _eq(tl.cpu().numpy(), rl)
    # fused kernel, one frame: planes 16-byte aligned, then 4-byte (offset 4), then unaligned (offset 1)
    for off, m in ((0, 1 << 24), (4, (1 << 24) - 16), (1, (1 << 20) - 1)):
        tf2 = torch.zeros(m + 16, dtype=torch.uint8, device=dev)
        tb2, tv2, tl2 = torch.zeros_like(tf2), torch.zeros_like(tf2), torch.zeros_like(tf2)
        tf2[off:off + m] = tf[:m]
        tb2[off:off + m] = _t(dev, b[:m])
        tv2[off:off + m] = _t(dev, v[:m])
        lib.sigmadelta_frames(tf2[off:off + m].view(1, m), tb2[off:off + m], tv2[off:off + m], tl2[off:off + m].view(1, m))
        torch.cuda.synchronize()
        assert _eq(tb2[off:off + m].cpu().numpy(), rb[:m]) and _eq(tv2[off:off + m].cpu().numpy(), rv[:m]), off
        assert _eq(tl2[off:off + m].cpu().numpy(), rl[:m]), off


@pytest.mark.parametrize("n", [1, 15, 17, 100003])
def test_sigmadelta_odd_sizes(lib, dev, oracle, n):
    rng = np.random.default_rng(n)
    f, b, v = (rng.integers(0, 256, n, dtype=np.uint8) for _ in range(3))
    tf, tb, tv = _t(dev, f), _t(dev, b), _t(dev, v)
    tl = torch.empty(n, dtype=torch.uint8, device=dev)
    lib.sigmadelta(tf, tb, tv, tl)
    torch.cuda.synchronize()
    rb, rv, rl = oracle.sigmadelta(f, b, v)
    assert _eq(tb.cpu().numpy(), rb) and _eq(tv.cpu().numpy(), rv) and _eq(tl.cpu().numpy(), rl)


def test_generic_interpreter_float_ops(lib, dev):
    n = 10007
    rng = np.random.default_rng(11)
    x, y = rng.uniform(0.5, 4, n).astype(np.float32), rng.uniform(-3, 3, n).astype(np.float32)
    tx, ty = _t(dev, x), _t(dev, y)
    X, Y = E.Table(tx), E.Table(ty)
    out = torch.empty_like(tx)
    e = E.if_else(X < Y, E.min_(X, Y) * 2.0, E.max_(X, Y) - E.rec(X)) + E.sqrt(X) / X - (-Y)
    prog = E.assign([out], [e], precision=lib.PREC_NT2)
    assert prog.info().kernel_name == b"generic"
    torch.cuda.synchronize()
    x32, y32 = x, y
    with np.errstate(all="ignore"):
        ref = np.where(x32 < y32, np.minimum(x32, y32) * np.float32(2), np.maximum(x32, y32) - np.float32(1) / x32)
        ref = (ref + np.sqrt(x32) / x32).astype(np.float32) - (-y32)
    assert _eq(out.cpu().numpy(), ref.astype(np.float32))


def test_generic_interpreter_uint8_wraparound(lib, dev):
    n = 4097
    rng = np.random.default_rng(12)
    a, b = rng.integers(0, 256, n, dtype=np.uint8), rng.integers(0, 256, n, dtype=np.uint8)
    ta, tb = _t(dev, a), _t(dev, b)
    A, B = E.Table(ta), E.Table(tb)
    o1, o2, o3 = (torch.empty_like(ta) for _ in range(3))
    E.assign([o1, o2, o3], [A + B, A - B, E.if_else(A >= B, E.adds(A, B), A * B)])
    torch.cuda.synchronize()
    assert _eq(o1.cpu().numpy(), (a + b).astype(np.uint8))
    assert _eq(o2.cpu().numpy(), (a - b).astype(np.uint8))
    sat = np.minimum(a.astype(int) + b, 255).astype(np.uint8)
    assert _eq(o3.cpu().numpy(), np.where(a >= b, sat, (a * b).astype(np.uint8)))
    # unary uint8 functors wrap the same way (sqr(a) = a*a mod 256), in both generic kernels
    for mode in (1, 2):
        E.assign([o1, o2, o3], [E.sqr(A), -A, E.abs_(B)], force_generic=mode)
        torch.cuda.synchronize()
        assert _eq(o1.cpu().numpy(), (a * a).astype(np.uint8)), mode
        assert _eq(o2.cpu().numpy(), (-a.astype(int)).astype(np.uint8)) and _eq(o3.cpu().numpy(), b), mode


def test_min_max_follow_nt2_operand_order(lib, dev):
    """max(a, b) = (a > b) ? a : b and min(a, b) = (a < b) ? a : b
    (boost/simd/arithmetic/functions/scalar/max.hpp, min.hpp): a NaN second
    operand wins, a NaN first operand loses, and -0/+0 ties take b."""
    a = np.array([1.0, np.nan, -0.0, 0.0, 2.0], np.float32)
    b = np.array([np.nan, 1.0, 0.0, -0.0, 2.0], np.float32)
    ta, tb = _t(dev, a), _t(dev, b)
    mx, mn = torch.empty_like(ta), torch.empty_like(ta)
    with np.errstate(invalid="ignore"):
        rmax, rmin = np.where(a > b, a, b), np.where(a < b, a, b)
    for mode in (1, 2):
        E.assign([mx, mn], [E.max_(E.Table(ta), E.Table(tb)), E.min_(E.Table(ta), E.Table(tb))], force_generic=mode)
        torch.cuda.synchronize()
        for got, ref in ((mx, rmax), (mn, rmin)):
            g = got.cpu().numpy()
            assert np.array_equal(np.isnan(g), np.isnan(ref)), mode
            assert np.array_equal(g[~np.isnan(g)].view(np.uint32), ref[~np.isnan(ref)].view(np.uint32)), mode


def test_logical_stored_into_float_table(lib, dev):
    x = np.array([1, 2, 3, 4, 5], np.float32)
    tx = _t(dev, x)
    out = torch.empty_like(tx)
    E.assign([out], [E.Table(tx) > 2.5])
    torch.cuda.synchronize()
    assert out.cpu().numpy().tolist() == [0, 0, 1, 1, 1]


@pytest.mark.parametrize("mode", [1, 2], ids=["compiled", "interpreter"])
def test_exp_log_family_in_expressions_nt2_policy(lib, dev, oracle, mode):
    """exp2(x) + exp10(y) * expm1(x - y) and log2(|x|) - log10(|y|) under NT2's
    policy, through the generic interpreter and the compiled kernel,
    bit-identical to the oracle's composition of the same rounded operations."""
    n = 100003
    rng = np.random.default_rng(21)
    x = rng.uniform(-30, 30, n).astype(np.float32)
    y = rng.uniform(-8, 8, n).astype(np.float32)
    x[:6] = [np.nan, np.inf, -np.inf, 127.0, -127.5, 0.0]
    tx, ty = _t(dev, x), _t(dev, y)
    X, Y = E.Table(tx), E.Table(ty)
    out, out2 = torch.empty_like(tx), torch.empty_like(tx)
    E.assign([out, out2], [E.exp2(X) + E.exp10(Y) * E.expm1(X - Y), E.log2(E.abs_(X)) - E.log10(E.abs_(Y))],
             precision=lib.PREC_NT2, force_generic=mode)
    torch.cuda.synchronize()
    with np.errstate(all="ignore"):
        ref = oracle.map_f32("exp2", x) + oracle.map_f32("exp10", y) * oracle.map_f32("expm1", (x - y).astype(np.float32))
        ref2 = oracle.map_f32("log2", np.abs(x)) - oracle.map_f32("log10", np.abs(y))
    for got, r in ((out.cpu().numpy(), ref), (out2.cpu().numpy(), ref2)):
        assert np.all((got.view(np.uint32) == r.view(np.uint32)) | (np.isnan(got) & np.isnan(r)))


@pytest.mark.parametrize("mode", [1, 2], ids=["compiled", "interpreter"])
def test_trig_in_expressions_nt2_policy(lib, dev, oracle, mode):
    """sin(x) * cos(y) + tan(x) - sinpi(y) * cospi(x) under NT2's policy through
    both generic paths, bit-identical to the oracle's composition."""
    n = 65537
    rng = np.random.default_rng(22)
    x = (rng.standard_normal(n) * np.exp2(rng.integers(-4, 22, n))).astype(np.float32)
    y = rng.uniform(-1e3, 1e3, n).astype(np.float32)
    tx, ty = _t(dev, x), _t(dev, y)
    X, Y = E.Table(tx), E.Table(ty)
    out = torch.empty_like(tx)
    E.assign([out], [E.sin(X) * E.cos(Y) + E.tan(X) - E.sinpi(Y) * E.cospi(X)], precision=lib.PREC_NT2,
             force_generic=mode)
    torch.cuda.synchronize()
    f = oracle.map_f32
    with np.errstate(all="ignore"):
        ref = (f("sin", x) * f("cos", y) + f("tan", x)) - f("sinpi", y) * f("cospi", x)
    got = out.cpu().numpy()
    assert np.all((got.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(got) & np.isnan(ref)))
