"""NT2's distribution functions (statistics/functions/generic/*.hpp) as NT2
composes them: normal pdf/inverse, exponential, lognormal, uniform, Cauchy and
extreme-value cdf/pdf/inverse (cauinv on proper_tanpi, NT2's tangent of pi x
restricted to [-1/2, 1/2]), with one- and multi-parameter forms.

NT2 policy: bit-identical to the same composition of the oracle's NT2 float
functors with float32 arithmetic in NT2's operation order.  Fast policy:
within max(4 x NT2's own distance from the FP64 value of the same formula,
16 ulp) + 8 ulp + 4 ulp x the formula's condition number (plus 1e-37), with
NT2's NaN positions: the compositions are ill-conditioned in places (a
difference inside erfc, fma(norminv(p), s, m) near -m/s, t exp(-t) for large
t), where an intermediate rounding moves both policies' results alike."""
import numpy as np
import pytest
import torch

from nt2_gb300 import expr as E

pytestmark = pytest.mark.gpu
F = np.float32
SQRT_2, SQRT_2O_2 = np.uint32(0x3fb504f3).view(F), np.uint32(0x3f3504f3).view(F)
INVSQRT_2PI, INVPI = np.uint32(0x3ecc422a).view(F), np.uint32(0x3ea2f983).view(F)


def _o(oracle, fn):
    return lambda x: oracle.map_f32(fn, np.asarray(x, F))


def cases(oracle, sp):
    """name -> (device composition, NT2 float32 composition, FP64 formula, input generator)."""
    exp, expm1, log, log1p = _o(oracle, "exp"), _o(oracle, "expm1"), _o(oracle, "log"), _o(oracle, "log1p")
    erfc, erfcinv, atan = _o(oracle, "erfc"), _o(oracle, "erfcinv"), _o(oracle, "atan")
    m, s, a, b = F(0.5), F(1.75), F(-1.25), F(2.5)
    rec = lambda v: (F(1) / v).astype(F)  # noqa: E731
    nan = F(np.nan)

    def normpdf3(x):
        inv = rec(s)
        return (exp(F(-0.5) * np.square((x - m) * inv)) * INVSQRT_2PI * inv).astype(F)

    def lognpdf3(x):
        xx = np.where(x <= 0, F(np.inf), x).astype(F)
        inv = rec(s)
        return (exp(F(-0.5) * np.square((log(xx) - m) * inv)) * INVSQRT_2PI * inv / xx).astype(F)

    def evpdf3(x):
        inv = rec(s)
        t = exp((x - m) * inv)
        t = (t * (exp(-t) * inv)).astype(F)
        return np.where(x == np.inf, F(0), t).astype(F)

    d = np.float64
    return {
        "normpdf": (lambda X: E.normpdf(X), lambda x: (exp(F(-0.5) * np.square(x)) * INVSQRT_2PI).astype(F),
                    lambda x: np.exp(-0.5 * x * x) / np.sqrt(2 * np.pi), "real"),
        "normpdf3": (lambda X: E.normpdf(X, float(m), float(s)), normpdf3,
                     lambda x: np.exp(-0.5 * ((x - d(m)) / d(s)) ** 2) / np.sqrt(2 * np.pi) / d(s), "real"),
        "norminv": (lambda X: E.norminv(X), lambda x: (-SQRT_2 * erfcinv(F(2) * x)).astype(F),
                    lambda x: -np.sqrt(2) * sp.erfcinv(2 * x), "prob"),
        "norminv3": (lambda X: E.norminv(X, float(m), float(s)), lambda x: (-SQRT_2 * erfcinv(F(2) * x) * s + m).astype(F),
                     lambda x: -np.sqrt(2) * sp.erfcinv(2 * x) * d(s) + d(m), "prob"),
        "expcdf": (lambda X: E.expcdf(X), lambda x: (-expm1(-np.where(x < 0, F(0), x).astype(F))).astype(F),
                   lambda x: -np.expm1(-np.where(x < 0, 0, x)), "real"),
        "expcdf2": (lambda X: E.expcdf(X, float(s)), lambda x: (-expm1(-np.where(x / s < 0, F(0), (x / s).astype(F)).astype(F))).astype(F),
                    lambda x: -np.expm1(-np.where(x < 0, 0, x / d(s))), "real"),
        "exppdf2": (lambda X: E.exppdf(X, float(s)), lambda x: np.where(x < 0, F(0), s * exp(-x * s)).astype(F),
                    lambda x: np.where(x < 0, 0, d(s) * np.exp(-x * d(s))), "real"),
        "expinv2": (lambda X: E.expinv(X, float(s)), lambda x: (s * np.where(x < 0, nan, -log1p(-x))).astype(F),
                    lambda x: d(s) * np.where(x < 0, np.nan, -np.log1p(-x)), "prob"),
        "logncdf3": (lambda X: E.logncdf(X, float(m), float(s)),
                     lambda x: (F(0.5) * erfc(SQRT_2O_2 * ((m - log(np.where(x <= 0, F(0), x).astype(F))) / s))).astype(F),
                     lambda x: 0.5 * sp.erfc(np.sqrt(0.5) * ((d(m) - np.log(np.where(x <= 0, 0, x))) / d(s))), "pos"),
        "lognpdf3": (lambda X: E.lognpdf(X, float(m), float(s)), lognpdf3,
                     lambda x: np.where(x <= 0, 0, np.exp(-0.5 * ((np.log(np.where(x <= 0, 1, x)) - d(m)) / d(s)) ** 2)
                                        / (np.sqrt(2 * np.pi) * d(s) * np.where(x <= 0, 1, x))), "pos"),
        "logninv3": (lambda X: E.logninv(X, float(m), float(s)),
                     lambda x: exp((-SQRT_2 * s) * erfcinv(F(2) * x) + m).astype(F),
                     lambda x: np.exp(-np.sqrt(2) * d(s) * sp.erfcinv(2 * x) + d(m)), "prob"),
        "unifcdf3": (lambda X: E.unifcdf(X, float(a), float(b)),
                     lambda x: np.where(x < a, F(0), np.where(x > b, F(1), ((x - a) / (b - a)).astype(F))).astype(F),
                     lambda x: np.clip((x - d(a)) / (d(b) - d(a)), 0, 1), "real"),
        "unifpdf": (lambda X: E.unifpdf(X),
                    lambda x: np.where(np.isnan(x), x, np.where((x <= 1) & ~np.signbit(x), F(1), F(0))).astype(F),
                    lambda x: np.where(np.isnan(x), x, np.where((x <= 1) & ~np.signbit(x), 1.0, 0.0)), "real"),
        "caucdf3": (lambda X: E.caucdf(X, float(m), float(s)),
                    lambda x: (F(0.5) + INVPI * atan(((x - m) / s).astype(F))).astype(F),
                    lambda x: 0.5 + np.arctan((x - d(m)) / d(s)) / np.pi, "real"),
        "proper_tanpi": (lambda X: E.proper_tanpi(X), lambda x: oracle.proper_tanpi_f32(x),
                         lambda x: np.where(np.abs(x) <= 0.5, np.tan(np.pi * x), np.nan), "half"),
        "cauinv": (lambda X: E.cauinv(X), lambda x: oracle.proper_tanpi_f32((x - F(0.5)).astype(F)),
                   lambda x: np.tan(np.pi * (x - 0.5)), "prob"),
        "cauinv3": (lambda X: E.cauinv(X, float(m), float(s)),
                    lambda x: ((oracle.proper_tanpi_f32((x - F(0.5)).astype(F)) * s).astype(F) + m).astype(F),
                    lambda x: np.tan(np.pi * (x - 0.5)) * d(s) + d(m), "prob"),
        "caupdf3": (lambda X: E.caupdf(X, float(m), float(s)),
                    lambda x: ((s * INVPI) / (s * s + np.square((x - m).astype(F)))).astype(F),
                    lambda x: d(s) / np.pi / (d(s) ** 2 + (x - d(m)) ** 2), "real"),
        "evcdf3": (lambda X: E.evcdf(X, float(m), float(s)), lambda x: (-expm1(-exp(((x - m) / s).astype(F)))).astype(F),
                   lambda x: -np.expm1(-np.exp((x - d(m)) / d(s))), "real"),
        "evpdf3": (lambda X: E.evpdf(X, float(m), float(s)), evpdf3,
                   lambda x: np.exp((x - d(m)) / d(s)) * np.exp(-np.exp((x - d(m)) / d(s))) / d(s), "real"),
        "evinv3": (lambda X: E.evinv(X, float(m), float(s)), lambda x: (log(-log1p(-x)) * s + m).astype(F),
                   lambda x: np.log(-np.log1p(-x)) * d(s) + d(m), "prob"),
    }


def _inputs(kind, rng):
    if kind == "prob":
        x = rng.uniform(0, 1, 1 << 15)
    elif kind == "half":
        x = rng.uniform(-0.5, 0.5, 1 << 15)
    elif kind == "pos":
        x = np.exp(rng.uniform(-8, 5, 1 << 15))
    else:
        x = rng.uniform(-8, 8, 1 << 15)
    extra = [0.0, -0.0, 1.0, -1.0, 0.5, np.inf, -np.inf, np.nan, 1e-30, 1 - 2 ** -24, 2.0, -3.0]
    return np.concatenate([x, extra]).astype(F)


@pytest.mark.parametrize("name", ["normpdf", "normpdf3", "norminv", "norminv3", "expcdf", "expcdf2", "exppdf2",
                                  "expinv2", "logncdf3", "lognpdf3", "logninv3", "unifcdf3", "unifpdf", "caucdf3",
                                  "proper_tanpi", "cauinv", "cauinv3", "caupdf3", "evcdf3", "evpdf3", "evinv3"])
@pytest.mark.parametrize("prec", [1, 0], ids=["nt2", "fast"])
def test_distribution(lib, dev, oracle, name, prec):
    sp = pytest.importorskip("scipy.special")
    dev_fn, nt2_fn, f64, kind = cases(oracle, sp)[name]
    rng = np.random.default_rng(abs(hash(name)) % (1 << 31))
    x = _inputs(kind, rng)
    tx = torch.from_numpy(x).to(dev)
    out = torch.empty_like(tx)
    E.assign([out], [dev_fn(E.Table(tx))], precision=prec)
    got = out.cpu().numpy()
    with np.errstate(all="ignore"):
        ref = nt2_fn(x)
        r64 = f64(x.astype(np.float64))
    same = (got.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(got) & np.isnan(ref))
    if prec == 1:
        assert same.all(), (name, x[~same][:4], got[~same][:4], ref[~same][:4])
        return
    assert np.array_equal(np.isnan(got), np.isnan(ref)), name
    ok = np.isfinite(r64) & np.isfinite(ref)
    sp32 = np.spacing(np.abs(r64[ok]).astype(F)).astype(np.float64)
    e_fast = np.abs(got[ok] - r64[ok]) / sp32
    e_nt2 = np.abs(ref[ok] - r64[ok]) / sp32
    # where a composition is ill-conditioned (fma(norminv(p), s, m) near -m/s,
    # t exp(-t) for large t, erfc of a difference) a rounding in an intermediate
    # value moves the result like a relative input perturbation of a few ulp:
    # bounded by 4 ulp times the formula's condition number |x f'(x) / f(x)|
    x64 = x[ok].astype(np.float64)
    h = 1e-6
    with np.errstate(all="ignore"):
        df = (f64(x64 * (1 + h)) - f64(x64 * (1 - h))) / (2 * h)
        kappa = np.nan_to_num(np.abs(df / r64[ok]), nan=0.0, posinf=1e30)
    bad = e_fast > np.maximum(4.0 * e_nt2, 16.0) + 8.0 + 4.0 * kappa + 1e-37 / sp32
    assert not bad.any(), (name, x[ok][bad][:4], e_fast[bad][:4], e_nt2[bad][:4])


STAT_FNS = ("normpdf", "norminv", "expcdf", "exppdf", "expinv", "logncdf", "lognpdf", "logninv", "unifcdf", "unifpdf",
            "unifinv", "caucdf", "cauinv", "caupdf", "evcdf", "evpdf", "evinv", "proper_tanpi")


@pytest.mark.parametrize("prec", [1, 0], ids=["nt2", "fast"])
def test_nt2_unit_answers(lib, dev, prec):
    """NT2's own known answers for the distribution functions (one- and
    two-argument forms, statistics/unit/scalar/*.cpp) in both policies."""
    import json
    import os
    from helpers import nt2_ulpdist
    golden = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "nt2_unit_vectors.json")))
    recs = [r for r in golden if r["fn"] in STAT_FNS]
    assert len(recs) >= 100
    for r in recs:
        tx = torch.tensor([r["x"]], dtype=torch.float32, device=dev)
        args = (E.Table(tx),) if "y" not in r else (E.Table(tx), float(r["y"]))
        out = torch.empty_like(tx)
        E.assign([out], [getattr(E, r["fn"])(*args)], precision=prec)
        got = float(out.cpu().numpy()[0])
        assert nt2_ulpdist(got, r["expected"]) <= (r["tol_nt2ulp"] if prec == 1 else max(r["tol_nt2ulp"], 4.0)), (r, got)
