"""The C++ table layer (nt2_gb300/include/nt2/table.hpp): NT2's demo
expressions, spelled as in the reference's demo sources, lower to programs
that bind the fused kernels (host-only), and produce the oracle's results on
the GPU through the C ABI."""
import os
import subprocess

import numpy as np
import pytest

from helpers import bs_inputs, sigmadelta_frames

HERE = os.path.dirname(os.path.abspath(__file__))
DEMOS = os.path.join(os.path.dirname(HERE), "nt2_gb300", "_build", "nt2_demos")


@pytest.fixture(scope="module")
def demos(lib):
    if not os.path.exists(DEMOS):
        from nt2_gb300 import build
        build.build_library()
    return DEMOS


def test_demo_expressions_bind_fused_kernels(demos):
    out = subprocess.run([demos, "lower"], check=True, capture_output=True, text=True).stdout.split("\n")
    got = dict(line.split() for line in out if line.strip())
    assert got == {"bs": "blackscholes", "bs_demo": "blackscholes_demo", "saxpy": "saxpy", "rgb2yuv": "rgb2yuv",
                   "sigmadelta": "sigmadelta"}


def _run(demos, *args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    r = subprocess.run([demos, *map(str, args)], capture_output=True, text=True, env=e)
    assert r.returncode == 0, f"nt2_demos {args[0]} exited {r.returncode}: {r.stderr.strip()}"
    return r.stdout


def _eq(a, b):
    return np.array_equal(np.asarray(a).view(np.uint8), np.asarray(b).view(np.uint8))


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["bs", "bs_host"])
def test_blackscholes_through_tables(demos, oracle, tmp_path, mode):
    n = 100003
    S, K, T = bs_inputs(n)
    for name, a in (("S", S), ("K", K), ("T", T)):
        a.tofile(tmp_path / f"{name}.bin")
    _run(demos, mode, tmp_path, n, env={"NT2G_PRECISION": "1"})
    rc, rp = oracle.blackscholes(S, K, T, 0.02, 0.30)
    assert _eq(np.fromfile(tmp_path / "call.bin", np.float32), rc)
    assert _eq(np.fromfile(tmp_path / "put.bin", np.float32), rp)


@pytest.mark.gpu
def test_blackscholes_demo_materialised_tables(demos, oracle, tmp_path):
    n = 65537
    S, X, T = bs_inputs(n)
    rng = np.random.default_rng(4)
    r = rng.uniform(0.01, 0.05, n).astype(np.float32)
    v = rng.uniform(0.1, 0.5, n).astype(np.float32)
    for name, a in (("S", S), ("K", X), ("T", T), ("r", r), ("v", v)):
        a.tofile(tmp_path / f"{name}.bin")
    _run(demos, "bs_demo", tmp_path, n, env={"NT2G_PRECISION": "1"})
    assert _eq(np.fromfile(tmp_path / "R.bin", np.float32), oracle.blackscholes_demo(S, X, T, r, v))


@pytest.mark.gpu
def test_saxpy_rgb2yuv_through_tables(demos, oracle, tmp_path):
    n = 1920 * 1080
    rng = np.random.default_rng(8)
    x, y = rng.standard_normal(n).astype(np.float32), rng.standard_normal(n).astype(np.float32)
    a = np.array([1.75], np.float32)
    x.tofile(tmp_path / "x.bin"); y.tofile(tmp_path / "y.bin"); a.tofile(tmp_path / "alpha.bin")
    _run(demos, "saxpy", tmp_path, n)
    assert _eq(np.fromfile(tmp_path / "y_out.bin", np.float32), oracle.saxpy(a[0], x, y))
    r, g, b = (rng.uniform(0, 1, n).astype(np.float32) for _ in range(3))
    for name, p in (("r", r), ("g", g), ("b", b)):
        p.tofile(tmp_path / f"{name}.bin")
    _run(demos, "rgb2yuv", tmp_path, n, env={"NT2G_PRECISION": "1"})
    for name, ref in zip("yuv", oracle.rgb2yuv(r, g, b)):
        assert _eq(np.fromfile(tmp_path / f"{name}.bin", np.float32), ref)


@pytest.mark.gpu
def test_sdot_through_tables(demos, oracle, tmp_path):
    n = 1 << 22
    rng = np.random.default_rng(9)
    x, y = rng.standard_normal(n).astype(np.float32), rng.standard_normal(n).astype(np.float32)
    x.tofile(tmp_path / "x.bin"); y.tofile(tmp_path / "y.bin")
    out = dict(line.split() for line in _run(demos, "sdot", tmp_path, n).splitlines())
    exact = oracle.exact_sum(x, y)[0]
    assert float(out["sum64"]) == pytest.approx(exact, rel=1e-13)
    assert np.float32(out["globalsum"]) == np.float32(exact) or abs(float(out["globalsum"]) - exact) <= abs(exact) * 1.2e-7
    assert float(out["sum"]) == pytest.approx(oracle.exact_sum(x)[0], rel=1e-6, abs=1e-3)
    ref = oracle.exact_sum(x * x + y)[0]  # x*x rounded to float first, as the kernel's temporary
    assert float(out["sum_expr"]) == pytest.approx(ref, rel=1e-6)


@pytest.mark.gpu
def test_sigmadelta_through_tables(demos, oracle, tmp_path):
    frames = sigmadelta_frames(h=540, w=960, frames=12, seed=21)
    F, H, W = frames.shape
    n = H * W
    frames.tofile(tmp_path / "frames.bin")
    _run(demos, "sigmadelta", tmp_path, n, F)
    rb, rv = frames[0].ravel().copy(), np.ones(n, np.uint8)
    for k in range(1, F):
        rb, rv, rl = oracle.sigmadelta(frames[k].ravel(), rb, rv)
    assert _eq(np.fromfile(tmp_path / "bkg.bin", np.uint8), rb)
    assert _eq(np.fromfile(tmp_path / "var.bin", np.uint8), rv)
    assert _eq(np.fromfile(tmp_path / "label.bin", np.uint8), rl)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["1", "0"], ids=["nt2", "fast"])
def test_folds_through_tables(demos, oracle, tmp_path, prec):
    """sum(A, 1), sum(A, 2), maximum/minimum/mean/norm2/var/stdev/meanad/
    median/medianad along a dimension, wmean, and the global forms of an M x N
    table through the C++ layer."""
    m, n = 1000, 777
    rng = np.random.default_rng(21)
    a = (rng.standard_normal(m * n) * np.exp2(rng.integers(-6, 6, m * n))).astype(np.float32)
    a.tofile(tmp_path / "a.bin")
    lines = _run(demos, "fold", tmp_path, m, n, env={"NT2G_PRECISION": prec}).splitlines()
    glob = {ln.split()[0]: ln.split()[1:] for ln in lines}
    cases = [("sum1", (1, m, n), "sum"), ("sum2", (m, n, 1), "sum"), ("max1", (1, m, n), "max"),
             ("min2", (m, n, 1), "min"), ("mean1", (1, m, n), "mean"), ("norm2_2", (m, n, 1), "norm2"),
             ("hsum1", (1, m, n), "sum"), ("var1", (1, m, n), "var"), ("stdev2_w1", (m, n, 1), "stdev1"),
             ("meanad1", (1, m, n), "meanad"), ("meanad2", (m, n, 1), "meanad")]
    for name, shape, op in cases:
        got = np.fromfile(tmp_path / f"{name}.bin", np.float32)
        if prec == "1":
            ref, _ = oracle.fold_nt2(a, *shape, op)
            assert _eq(got, ref), name
        else:
            ref, _, _ = oracle.fold_ref(a, *shape, op)
            k = 2.0 if op in ("var", "stdev1", "meanad") else 1.0
            assert (np.abs(got - ref) <= k * np.spacing(np.abs(ref).astype(np.float32))).all(), name
    # wmean(A, abs(A), 1) = rec(globalsum(w)) * sum(A .* w, 1)
    w = np.abs(a)
    wm = np.fromfile(tmp_path / "wmean1.bin", np.float32)
    if prec == "1":
        # the layer's globalsum is the compensated device reduction (the float
        # nearest the exact sum, give or take one rounding), the fold along
        # the dimension NT2's in-order one
        f = np.float32(1.0) / np.float32(oracle.exact_sum(w)[0])
        ref = (f * oracle.fold_nt2((a * w).astype(np.float32), 1, m, n, "sum")[0]).astype(np.float32)
        assert (np.abs(wm - ref) <= np.spacing(np.abs(ref))).all()
    else:
        gw = oracle.fold_ref(w, 1, m * n, 1, "sum")[0][0]
        s, sa, _ = oracle.fold_ref((a * w).astype(np.float32), 1, m, n, "sum")
        ref = s / gw
        assert (np.abs(wm - ref) <= 2 * np.spacing(np.abs(ref).astype(np.float32)) + 2e-7 * sa / gw).all()
    c1 = np.fromfile(tmp_path / "cumsum1.bin", np.float32)
    c2 = np.fromfile(tmp_path / "cummax2.bin", np.float32)
    assert _eq(c2, oracle.scan_nt2(a, m, n, 1, "max"))
    if prec == "1":
        assert _eq(c1, oracle.scan_nt2(a, 1, m, n, "sum"))
    else:
        ref, absrun = oracle.cumsum_exact(a, 1, m, n)
        assert (np.abs(c1 - ref) <= np.spacing(np.abs(ref).astype(np.float32)) + 1e-12 * absrun).all()
    gmax, imax = oracle.fold_nt2(a, 1, m * n, 1, "max")
    gmin, imin = oracle.fold_nt2(a, 1, m * n, 1, "min")
    assert np.float32(glob["globalmax"][0]) == gmax[0] and int(glob["globalmax"][1]) == imax[0] + 1
    assert np.float32(glob["globalmin"][0]) == gmin[0] and int(glob["globalmin"][1]) == imin[0] + 1
    for key, op in (("globalmean", "mean"), ("globalnorm2", "norm2"), ("globalasum1", "asum1"), ("globalvar", "var"),
                    ("globalstdev", "stdev")):
        if prec == "1":
            ref, _ = oracle.fold_nt2(a, 1, m * n, 1, op)
            assert np.float32(glob[key][0]) == ref[0], key
        else:
            ref, _, _ = oracle.fold_ref(a, 1, m * n, 1, op)
            assert abs(float(glob[key][0]) - ref[0]) <= 2 * np.spacing(np.float32(abs(ref[0]))), key
    # median(A, 1), median(h, 2) of the host table, medianad(A) and the global
    # forms: the same order statistics under either policy
    for name, shape, ad in (("median1", (1, m, n), False), ("median2", (m, n, 1), False),
                            ("medianad1", (1, m, n), True)):
        got = np.fromfile(tmp_path / f"{name}.bin", np.float32)
        assert np.array_equal(got, oracle.median(a, *shape, ad=ad)), name
    assert np.float32(glob["globalmedian"][0]) == oracle.median(a, 1, m * n, 1)[0]
    assert np.float32(glob["globalmedianad"][0]) == oracle.median(a, 1, m * n, 1, ad=True)[0]
    # asump(A, 3, 1) = sum(pow(abs(A), 3), 1), normp(h, 1.5, 2) = pow(asump(h, 1.5, 2), rec(1.5)), and
    # the global forms (globalasump a compensated global sum)
    p3, p15 = np.float32(3.0), np.float32(1.5)
    a3 = oracle.pow_f32(np.abs(a), np.full_like(a, p3))
    a15 = oracle.pow_f32(np.abs(a), np.full_like(a, p15))
    inv15 = np.float32(1.0) / p15
    got_as = np.fromfile(tmp_path / "asump1.bin", np.float32)
    got_np = np.fromfile(tmp_path / "normp2.bin", np.float32)
    a64 = np.abs(a.astype(np.float64))
    if prec == "1":
        assert _eq(got_as, oracle.fold_nt2(a3, 1, m, n, "sum")[0])
        s15 = oracle.fold_nt2(a15, m, n, 1, "sum")[0]
        assert _eq(got_np, oracle.pow_f32(s15, np.full_like(s15, inv15)))
        ga = np.float32(glob["globalasump"][0])
        assert abs(float(ga) - oracle.exact_sum(a3)[0]) <= np.spacing(ga)  # NT2's elements, compensated sum
        gs = np.float32([oracle.exact_sum(a15)[0]])
        gn = oracle.pow_f32(gs, np.float32([inv15]))[0]  # NT2's pow of the (float-nearest) sum
        assert abs(np.float32(glob["globalnormp"][0]) - gn) <= 2 * np.spacing(gn)
    else:
        # positive terms each within 4 ulp: sums within 5, their 1/1.5 roots within 4 + 5/1.5
        ref = (a64 ** 3).reshape(n, m).sum(axis=1)
        assert (np.abs(got_as - ref) <= 5 * np.spacing(ref.astype(np.float32))).all()
        ref = ((a64 ** 1.5).reshape(n, m).sum(axis=0)) ** (1 / 1.5)
        assert (np.abs(got_np - ref) <= 8 * np.spacing(ref.astype(np.float32))).all()
        ga = (a64 ** 3).sum()
        assert abs(float(glob["globalasump"][0]) - ga) <= 5 * np.spacing(np.float32(ga))
        gn = (a64 ** 1.5).sum() ** (1 / 1.5)
        assert abs(float(glob["globalnormp"][0]) - gn) <= 8 * np.spacing(np.float32(gn))
    # nanasum2(A, 2) = sum(is_nan(A) ? 0 : A*A, 2); globalmeanad, globalnorm(h, inf), globalnorm(A, 1)
    sq = np.where(np.isnan(a), np.float32(0), (a * a).astype(np.float32)).astype(np.float32)
    got = np.fromfile(tmp_path / "nanasum2_2.bin", np.float32)
    if prec == "1":
        assert _eq(got, oracle.fold_nt2(sq, m, n, 1, "sum")[0])
        assert np.float32(glob["globalmeanad"][0]) == oracle.fold_nt2(a, 1, m * n, 1, "meanad")[0][0]
        assert np.float32(glob["globalnorm_1"][0]) == oracle.fold_nt2(a, 1, m * n, 1, "asum1")[0][0]
    else:
        ref, _, _ = oracle.fold_ref(sq, m, n, 1, "sum")
        assert (np.abs(got - ref) <= np.spacing(np.abs(ref).astype(np.float32))).all()
        ref = oracle.fold_ref(a, 1, m * n, 1, "meanad")[0][0]
        assert abs(float(glob["globalmeanad"][0]) - ref) <= 2 * np.spacing(np.float32(abs(ref)))
        ref = oracle.fold_ref(a, 1, m * n, 1, "asum1")[0][0]
        assert abs(float(glob["globalnorm_1"][0]) - ref) <= np.spacing(np.float32(abs(ref)))
    assert np.float32(glob["globalnorm_inf"][0]) == np.abs(a).max()
    # trapz(A) along the first dimension, trapz(h, 2) of the host table along the rows
    for name, shape in (("trapz1", (1, m, n)), ("trapz2", (m, n, 1))):
        got = np.fromfile(tmp_path / f"{name}.bin", np.float32)
        if prec == "1":
            assert _eq(got, oracle.trapz_nt2(a, *shape)), name
        else:
            lo, inner, hi = shape
            v = a.astype(np.float64).reshape(hi, inner, lo)
            ref = (0.5 * (v[:, 1:, :] + v[:, :-1, :]).sum(axis=1)).ravel()
            mag = np.abs(v).sum(axis=1).ravel()
            assert (np.abs(got - ref) <= np.spacing(np.abs(ref).astype(np.float32)) + 2e-7 * mag).all(), name


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["1", "0"], ids=["nt2", "fast"])
def test_generative_through_tables(demos, oracle, tmp_path, prec):
    """_(0, 9), _(0, 0.3, 1), colon(1, -0.3, 0), linspace, logspace (with its
    pi rule), sinpi(linspace(0, 2, n)) * colon(1, n) + ones(1, n) and
    zeros(3) + 2 through the C++ layer:
    NT2's sizes, and under the NT2 policy NT2's values bit for bit."""
    n = 100003
    sizes = [int(v) for v in _run(demos, "gen", tmp_path, n, env={"NT2G_PRECISION": prec}).split()]
    pos = np.arange(n, dtype=np.float32)
    want = dict(c1=oracle.colon_nt2(0, 9), c2=oracle.colon_nt2(0, 0.3, 1), c3=oracle.colon_nt2(1, -0.3, 0),
                l1=oracle.linspace_nt2(-1, 1, 257), l2=oracle.linspace_nt2(0, 1), g1=oracle.logspace_nt2(0, 1),
                g2=oracle.logspace_nt2(2, np.float32(np.pi), 7),
                w=oracle.map_f32("sinpi", oracle.linspace_nt2(0, 2, n)) * (pos + np.float32(1)) + np.float32(1),
                o1=np.full(9, 2.0, np.float32))
    assert sizes == [len(v) for v in want.values()]
    for name, ref in want.items():
        got = np.fromfile(tmp_path / f"{name}.bin", np.float32)
        if prec == "1" or name in ("c1", "l1"):  # integers and dyadic steps are exact either way
            assert _eq(got, ref.astype(np.float32)), name
        else:
            # fused fma moves a colon/linspace value by at most half an ulp; exp10
            # amplifies that by ln(10)|x| and the fast exp10 differs by ~2.5 ulp;
            # sinpi near its zeros turns it into ~pi/2 ulp(x) <= 4e-7, times (p + 1)
            ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
            if name == "w":
                tol = 4 * ulp + (pos.astype(np.float64) + 1) * 1e-6 + 1.2e-7
            else:
                tol = {"g1": 4, "g2": 8}.get(name, 1) * ulp
            assert (np.abs(got.astype(np.float64) - ref) <= tol).all(), name


def _gpu_tensor(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0")


@pytest.mark.gpu
def test_expression_folds_through_tables(demos, lib, tmp_path):
    """sum(abs(A - B), 1), maximum(exp(A) - B, 2), var(A*B + 1, 0, 1),
    globalmax(A*B + 1, i), sum64(exp(A)*B) and globalmean(abs(A - B)) through
    the C++ table layer: each folds its expression in one pass, and equals the
    same fold through the C ABI from Python bit for bit."""
    from nt2_gb300 import expr as E
    m, n = 1000, 300
    rng = np.random.default_rng(31)
    a, b = rng.standard_normal(m * n).astype(np.float32), rng.standard_normal(m * n).astype(np.float32)
    a.tofile(tmp_path / "a.bin"); b.tofile(tmp_path / "b.bin")
    out = dict((ln.split()[0], ln.split()[1:]) for ln in _run(demos, "fold_expr", tmp_path, m, n).splitlines())
    A, B = E.Table(_gpu_tensor(a)), E.Table(_gpu_tensor(b))
    f32 = lambda p: np.fromfile(tmp_path / p, np.float32)  # noqa: E731
    assert _eq(f32("sumabs1.bin"), E.fold(E.abs_(A - B), "sum", (1, m, n)).cpu().numpy())
    assert _eq(f32("maxexp2.bin"), E.fold(E.exp(A) - B, "max", (m, n, 1)).cpu().numpy())
    assert _eq(f32("var1.bin"), E.fold(A * B + 1.0, "var", (1, m, n)).cpu().numpy())
    v, i = E.fold(A * B + 1.0, "max", index=True)
    assert np.float32(out["globalmax"][0]) == v.item() and int(out["globalmax"][1]) == i.item() + 1
    _, s64 = E.fold(E.exp(A) * B, "sum", out64=True)
    assert float(out["globalsum"][0]) == s64.item()
    assert np.float32(out["globalmean"][0]) == E.fold(E.abs_(A - B), "mean").item()
    np.testing.assert_allclose(f32("sumabs1.bin"), np.abs(a - b).reshape(n, m).astype(np.float64).sum(1), rtol=1e-6)


@pytest.mark.gpu
def test_reductions_from_two_host_threads(demos, lib, tmp_path):
    """Two host threads, each on its own stream with its own per-thread
    scratch, reduce concurrently (plain sum, dot, a fused expression sum): 40
    repetitions reproduce each thread's first results, which equal the same
    reductions through the C ABI."""
    from nt2_gb300 import expr as E
    n = 1 << 22
    rng = np.random.default_rng(32)
    x, y = rng.standard_normal(n).astype(np.float32), rng.standard_normal(n).astype(np.float32)
    x.tofile(tmp_path / "x.bin"); y.tofile(tmp_path / "y.bin")
    lines = _run(demos, "threads", tmp_path, n).splitlines()
    red = lib.Reducer("cuda:0")
    for tid, ln in enumerate(lines):
        r0, r1, r2, bad = ln.split()
        assert int(bad) == 0
        tx, ty = _gpu_tensor(x * np.float32(tid + 1)), _gpu_tensor(y + np.float32(tid))
        assert float(r0) == red(tx)[0].item()
        assert float(r1) == red(tx, ty)[0].item()
        assert float(r2) == E.fold(E.exp(E.Table(ty)) * E.Table(tx), "sum", out64=True)[1].item()


@pytest.mark.gpu
def test_async_sums_on_two_streams(demos, lib, tmp_path):
    """sum64_async in flight on two streams at once (per-stream scratch): 16
    dot products on one stream and 16 fused expression sums on the other all
    equal their single-stream values."""
    from nt2_gb300 import expr as E
    n = 1 << 22
    rng = np.random.default_rng(33)
    x, y = rng.standard_normal(n).astype(np.float32), rng.standard_normal(n).astype(np.float32)
    x.tofile(tmp_path / "x.bin"); y.tofile(tmp_path / "y.bin")
    vals = [float(v) for v in _run(demos, "streams", tmp_path, n).split()]
    tx, ty = _gpu_tensor(x), _gpu_tensor(y)
    dot = lib.Reducer("cuda:0")(tx, ty)[0].item()
    fused = E.fold(E.exp(E.Table(tx)) * E.Table(ty), "sum", out64=True)[1].item()
    assert vals[:16] == [dot] * 16 and vals[16:] == [fused] * 16


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["1", "0"], ids=["nt2", "fast"])
def test_distribution_functions_through_tables(demos, tmp_path, prec):
    """NT2's distribution functions through the C++ layer (parameters as
    numbers, resolved on the host where NT2's selects test them) give the same
    bits as the Python front end's compositions (parameters as run-time
    scalars) under the same policy."""
    import torch
    from nt2_gb300 import expr as E
    n = 50000
    rng = np.random.default_rng(81)
    x = np.concatenate([rng.uniform(-6, 6, n - 8), [0, -0.0, 1, -1, np.inf, -np.inf, np.nan, 2.5]]).astype(np.float32)
    p = np.concatenate([rng.uniform(0, 1, n - 6), [0, 1, -0.5, 1.5, np.nan, 0.5]]).astype(np.float32)
    x.tofile(tmp_path / "x.bin")
    p.tofile(tmp_path / "p.bin")
    _run(demos, "stat", tmp_path, n, env={"NT2G_PRECISION": prec})
    tx, tp = torch.from_numpy(x).cuda(), torch.from_numpy(p).cuda()
    X, P = E.Table(tx), E.Table(tp)
    m, s = 0.5, 1.75
    cases = {"normpdf3": E.normpdf(X, m, s), "norminv3": E.norminv(P, m, s), "expcdf2": E.expcdf(X, s),
             "exppdf2": E.exppdf(X, s), "expinv2": E.expinv(P, s), "logncdf3": E.logncdf(X, m, s),
             "lognpdf3": E.lognpdf(X, m, s), "logninv3": E.logninv(P, m, s), "unifcdf3": E.unifcdf(X, -1.25, 2.5),
             "unifpdf": E.unifpdf(X), "unifinv": E.unifinv(P), "caucdf3": E.caucdf(X, m, s),
             "caupdf3": E.caupdf(X, m, s), "evcdf3": E.evcdf(X, m, s), "evpdf3": E.evpdf(X, m, s),
             "evinv3": E.evinv(P, m, s), "cauinv3": E.cauinv(P, m, s), "cauinv2": E.cauinv(P, m),
             "maxnum": E.maxnum(X, P), "minnum": E.minnum(P, X), "maxmag": E.maxmag(X, P), "minmag": E.minmag(X, P),
             "minmod": E.minmod(X, P - 0.5), "negate": E.negate(P, X), "fms": E.fms(X, P, 0.25),
             "fnma": E.fnma(X, P, X), "divfloor": E.divfloor(X, P), "divround2even": E.divround2even(X, 0.75),
             "one_param_sum": (E.normpdf(X) + E.norminv(P) + E.expcdf(X) + E.exppdf(X) + E.expinv(P) + E.logncdf(X)
                               + E.lognpdf(X) + E.logninv(P) + E.unifcdf(X) + E.caucdf(X) + E.caupdf(X) + E.evcdf(X)
                               + E.evpdf(X) + E.evinv(P) + E.cauinv(P))}
    for name, e in cases.items():
        out = torch.empty_like(tx)
        E.assign([out], [e], precision=int(prec))
        want = out.cpu().numpy()
        got = np.fromfile(tmp_path / f"{name}.bin", np.float32)
        same = (got.view(np.uint32) == want.view(np.uint32)) | (np.isnan(got) & np.isnan(want))
        assert same.all(), (name, x[~same][:3], p[~same][:3], got[~same][:3], want[~same][:3])
