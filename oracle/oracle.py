"""TEST INFRASTRUCTURE ONLY -- loader for the CPU oracle (nt2_oracle.c).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker and as the timed CPU baseline.  The product library
never links, loads or calls it.

The reference itself cannot be built here (it needs Boost >= 1.59 and
configure-time generated headers), so there is no oracle/_ref; the oracle is
the restatement in nt2_oracle.c, pinned against NT2's unit-test golden values
(tests/golden/nt2_unit_vectors.json).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "_build", "liboracle.so")
SRC = os.path.join(HERE, "nt2_oracle.c")

FN = dict(exp=0, log=1, log1p=2, erfc=3, normcdf=4, fastnormcdf=5, sqrt=6, exp2=8, exp10=9, expm1=10, log2=11, log10=12,
          sin=13, cos=14, tan=15, sinpi=16, cospi=17, sinh=18, cosh=19, tanh=20, asin=21, acos=22, atan=23,
          asinh=24, acosh=25, atanh=26, cbrt=27, cot=28, sec=29, csc=30, sind=31, cosd=32, tand=33,
          tanpi=34, cotpi=35, cotd=36, secpi=37, cscpi=38, secd=39, cscd=40, sinc=41, sincpi=42, acotd=43, asec=44,
          coth=45, sinhc=46, acsc=47, asech=48, acoth=49, acsch=50,
          # NT2's generic compositions of the functors above
          sech=51, csch=52, acot=53, asind=54, acosd=55, atand=56, asecd=57, acscd=58, asinpi=59, acospi=60,
          atanpi=61, indeg=62, inrad=63,
          erf=64, erfcx=65, expx2=66, gamma=67, gammaln=68, erfinv=69, erfcinv=70, digamma=71, signgam=72, dawson=73, spence=74, stirling=75,
          exprecneg=80, exprecnegc=81, sqrt1pm1=82)
SCALAR_ONLY = ("o_realsqrt", "o_reallog", "o_floor", "o_ceil", "o_trunc", "o_fix", "o_round", "o_round2even",
               "o_frac", "o_sign", "o_signnz", "o_oneplus", "o_oneminus", "o_minusone", "o_sqr_abs", "o_proper_tanpi")


def build():
    os.makedirs(os.path.dirname(SO), exist_ok=True)
    if os.path.exists(SO) and os.path.getmtime(SO) >= os.path.getmtime(SRC):
        return SO
    # -ffp-contract=off: NT2's fma/fnms/Horner are unfused (two roundings)
    subprocess.run(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
                    "-shared", "-o", SO, SRC, "-lm"], check=True)
    return SO


_L = None
_P = ctypes.c_void_p
_I64 = ctypes.c_int64


def lib():
    global _L
    if _L is None:
        build()
        L = ctypes.CDLL(SO)
        for f in ("o_exp", "o_log", "o_log1p", "o_erfc", "o_normcdf", "o_fastnormcdf", "o_exp2", "o_exp10", "o_expm1",
                  "o_log2", "o_log10", "o_sin", "o_cos", "o_tan", "o_sinpi", "o_cospi",
                  "o_sinh", "o_cosh", "o_tanh", "o_asin", "o_acos", "o_atan",
                  "o_asinh", "o_acosh", "o_atanh", "o_cbrt", "o_cot", "o_sec", "o_csc", "o_sind", "o_cosd", "o_tand",
                  *("o_" + k for k, v in FN.items() if v >= 34), *SCALAR_ONLY):
            getattr(L, f).restype = ctypes.c_float
            getattr(L, f).argtypes = [ctypes.c_float]
        L.o_map_f32.argtypes = [ctypes.c_int, _P, _P, _I64]
        L.o_pow.restype = ctypes.c_float
        L.o_pow.argtypes = [ctypes.c_float, ctypes.c_float]
        L.o_pow_f32.argtypes = [_P, _P, _P, _I64]
        L.o_pow_f64.argtypes = [_P, _P, _P, _I64]
        L.o_atan2.restype = ctypes.c_float
        L.o_atan2.argtypes = [ctypes.c_float, ctypes.c_float]
        L.o_atan2_f32.argtypes = [_P, _P, _P, _I64]
        L.o_atan2_f64.argtypes = [_P, _P, _P, _I64]
        for f in ("o_logspace_add", "o_logspace_sub", "o_copysign", "o_dist", "o_average", "o_beta", "o_betaln",
                  "o_mod", "o_rem", "o_pow2", "o_maxnum", "o_minnum", "o_maxmag", "o_minmag", "o_minmod",
                  "o_negate", "o_divfloor", "o_divceil", "o_divfix", "o_divround", "o_divround2even"):
            getattr(L, f).restype = ctypes.c_float
            getattr(L, f).argtypes = [ctypes.c_float, ctypes.c_float]
        L.o_nthroot.restype = ctypes.c_float
        L.o_nthroot.argtypes = [ctypes.c_float, ctypes.c_int32]
        L.o_expni.restype = ctypes.c_float
        L.o_expni.argtypes = [ctypes.c_int32, ctypes.c_float]
        L.o_nthroot_f32.argtypes = [_P, _P, _P, _I64]
        L.o_expni_f32.argtypes = [_P, _P, _P, _I64]
        L.o_proper_tanpi_f32.argtypes = [_P, _P, _I64]
        L.o_atan2d.restype = ctypes.c_float
        L.o_atan2d.argtypes = [ctypes.c_float, ctypes.c_float]
        L.o_hypot.restype = ctypes.c_float
        L.o_hypot.argtypes = [ctypes.c_float, ctypes.c_float]
        L.o_hypot_f32.argtypes = [_P, _P, _P, _I64]
        L.o_hypot_f64.argtypes = [_P, _P, _P, _I64]
        L.o_map_f64.argtypes = [ctypes.c_int, _P, _P, _I64]
        L.o_bs_f32.argtypes = [_P, _P, _P, _P, ctypes.c_float, _P, ctypes.c_float, _P, _P, _I64, ctypes.c_int]
        L.o_bs_demo_f32.argtypes = [_P, _P, _P, _P, ctypes.c_float, _P, ctypes.c_float, _P, _I64, ctypes.c_int]
        L.o_bs_f64.argtypes = [_P, _P, _P, _P, ctypes.c_float, ctypes.c_float, _P, _P, _P, _I64]
        L.o_bs_vjp_f64.argtypes = [_P, _P, _P, _P, ctypes.c_float, ctypes.c_float, _P, _P, _P, _P, _P, _P, _P, _I64]
        L.o_bs_vjp_scale_f64.argtypes = [_P, _P, _P, _P, ctypes.c_float, ctypes.c_float, _P, _P, _P, _P, _P, _P,
                                          _P, _I64]
        L.o_bs_point_f64.argtypes = [ctypes.c_double] * 5 + [_P, _P]
        L.o_saxpy_f32.argtypes = [ctypes.c_float, _P, _P, _I64, ctypes.c_int]
        L.o_expr3_f32.argtypes = [_P, _P, _P, _P, _I64, ctypes.c_int]
        L.o_expr3_f64.argtypes = [_P, _P, _P, _P, _I64]
        L.o_rgb2yuv_f32.argtypes = [_P, _P, _P, _P, _P, _P, _I64, ctypes.c_int]
        L.o_sigmadelta_u8.argtypes = [_P, _P, _P, _P, _I64, ctypes.c_int]
        L.o_sum_nt2_f32.restype = ctypes.c_float
        L.o_sum_nt2_f32.argtypes = [_P, _P, _I64, ctypes.c_int]
        L.o_sum_plain_f32.restype = ctypes.c_float
        L.o_sum_plain_f32.argtypes = [_P, _P, _I64, ctypes.c_int]
        L.o_fold_nt2_f32.argtypes = [_P, _I64, _I64, _I64, ctypes.c_int, _P, _P, ctypes.c_int]
        L.o_fold_ref.argtypes = [_P, _I64, _I64, _I64, ctypes.c_int, _P, _P, _P, ctypes.c_int]
        L.o_median_f32.argtypes = [_P, _I64, _I64, _I64, ctypes.c_int, _P]
        L.o_trapz_nt2_f32.argtypes = [_P, _I64, _I64, _I64, _P]
        L.o_scan_nt2_f32.argtypes = [_P, _I64, _I64, _I64, ctypes.c_int, _P, ctypes.c_int]
        L.o_cumsum_exact.argtypes = [_P, _I64, _I64, _I64, _P, _P, ctypes.c_int]
        L.o_globalsum_f32.restype = ctypes.c_float
        L.o_globalsum_f32.argtypes = [_P, _I64]
        L.o_exact_sum.restype = ctypes.c_double
        L.o_exact_sum.argtypes = [_P, _P, _I64, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        L.o_nt2_transform_grain.restype = _I64
        L.o_nt2_transform_grain.argtypes = [_I64]
        L.o_max_threads.restype = ctypes.c_int
        _L = L
    return _L


def _p(a):
    return None if a is None else a.ctypes.data_as(_P)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def map_f32(fn, x):
    x = _f32(x)
    y = np.empty_like(x)
    lib().o_map_f32(FN[fn], _p(x), _p(y), x.size)
    return y


def map_f64(fn, x):
    x = _f32(x)
    y = np.empty(x.shape, np.float64)
    lib().o_map_f64(FN[fn], _p(x), _p(y), x.size)
    return y


def pow_f32(x, y):
    """NT2's float pow restated (Cephes powf with NT2's special cases)."""
    x, y = np.broadcast_arrays(_f32(x), _f32(y))
    x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
    out = np.empty(x.size, np.float32)
    lib().o_pow_f32(_p(x), _p(y), _p(out), x.size)
    return out


def pow_f64(x, y):
    x, y = np.broadcast_arrays(_f32(x), _f32(y))
    x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
    out = np.empty(x.size, np.float64)
    lib().o_pow_f64(_p(x), _p(y), _p(out), x.size)
    return out


def nthroot_f32(x, n):
    """NT2's float nthroot(x, n) restated, n given as floats (truncated)."""
    x, n = _f32(x), _f32(n)
    out = np.empty_like(x)
    lib().o_nthroot_f32(_p(x), _p(n), _p(out), x.size)
    return out


def proper_tanpi_f32(x):
    """NT2's float proper_tanpi(x) restated (tan(pi x) on [-1/2, 1/2])."""
    x = _f32(x)
    out = np.empty_like(x)
    lib().o_proper_tanpi_f32(_p(x), _p(out), x.size)
    return out


def expni_f32(n, x):
    """NT2's float expni(n, x) restated, n given as floats (truncated)."""
    n, x = _f32(n), _f32(x)
    out = np.empty_like(x)
    lib().o_expni_f32(_p(n), _p(x), _p(out), x.size)
    return out


def atan2_f32(x, y):
    """NT2's float atan2 restated."""
    x, y = np.broadcast_arrays(_f32(x), _f32(y))
    x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
    out = np.empty(x.size, np.float32)
    lib().o_atan2_f32(_p(x), _p(y), _p(out), x.size)
    return out


def atan2_f64(x, y):
    x, y = np.broadcast_arrays(_f32(x), _f32(y))
    x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
    out = np.empty(x.size, np.float64)
    lib().o_atan2_f64(_p(x), _p(y), _p(out), x.size)
    return out


def hypot_f32(x, y):
    """NT2's float hypot restated."""
    x, y = np.broadcast_arrays(_f32(x), _f32(y))
    x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
    out = np.empty(x.size, np.float32)
    lib().o_hypot_f32(_p(x), _p(y), _p(out), x.size)
    return out


def hypot_f64(x, y):
    x, y = np.broadcast_arrays(_f32(x), _f32(y))
    x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
    out = np.empty(x.size, np.float64)
    lib().o_hypot_f64(_p(x), _p(y), _p(out), x.size)
    return out


def threads():
    return lib().o_max_threads()


def blackscholes(S, K, T, r, sigma, nthreads=None):
    """NT2 restatement (float), textbook call+put; sigma scalar or array."""
    S, K, T = _f32(S), _f32(K), _f32(T)
    call, put = np.empty_like(S), np.empty_like(S)
    sig_t = _f32(sigma) if isinstance(sigma, np.ndarray) else None
    lib().o_bs_f32(_p(S), _p(K), _p(T), _p(sig_t), 0.0 if sig_t is not None else float(sigma), None, float(r),
                   _p(call), _p(put), S.size, nthreads or threads())
    return call, put


def blackscholes_f64(S, K, T, r, sigma):
    S, K, T = _f32(S), _f32(K), _f32(T)
    call, put = np.empty(S.shape), np.empty(S.shape)
    terms = np.empty((S.size, 4))
    sig_t = _f32(sigma) if isinstance(sigma, np.ndarray) else None
    lib().o_bs_f64(_p(S), _p(K), _p(T), _p(sig_t), 0.0 if sig_t is not None else float(sigma), float(r),
                   _p(call), _p(put), _p(terms), S.size)
    return call, put, terms


def blackscholes_demo(S, X, T, r, v, nthreads=None):
    S, X, T = _f32(S), _f32(X), _f32(T)
    R = np.empty_like(S)
    r_t = _f32(r) if isinstance(r, np.ndarray) else None
    v_t = _f32(v) if isinstance(v, np.ndarray) else None
    lib().o_bs_demo_f32(_p(S), _p(X), _p(T), _p(r_t), 0.0 if r_t is not None else float(r), _p(v_t),
                        0.0 if v_t is not None else float(v), _p(R), S.size, nthreads or threads())
    return R


def blackscholes_vjp_f64(S, K, T, sigma, r, gc, gp):
    S, K, T, sigma, gc, gp = (_f32(a) for a in (S, K, T, sigma, gc, gp))
    outs = [np.empty(S.shape) for _ in range(5)]
    lib().o_bs_vjp_f64(_p(S), _p(K), _p(T), _p(sigma), 0.0, float(r), _p(gc), _p(gp), *[_p(o) for o in outs],
                       S.size)
    return outs


def blackscholes_vjp_scale_f64(S, K, T, sigma, r, gc, gp):
    S, K, T, sigma, gc, gp = (_f32(a) for a in (S, K, T, sigma, gc, gp))
    outs = [np.empty(S.shape) for _ in range(5)]
    lib().o_bs_vjp_scale_f64(_p(S), _p(K), _p(T), _p(sigma), 0.0, float(r), _p(gc), _p(gp),
                             *[_p(o) for o in outs], S.size)
    return outs


def blackscholes_point_f64(s, k, t, v, r):
    c, p = ctypes.c_double(), ctypes.c_double()
    lib().o_bs_point_f64(s, k, t, v, r, ctypes.byref(c), ctypes.byref(p))
    return c.value, p.value


def saxpy(alpha, X, Y, nthreads=None):
    X, Y = _f32(X), _f32(Y).copy()
    lib().o_saxpy_f32(float(alpha), _p(X), _p(Y), X.size, nthreads or threads())
    return Y


def expr3(x, y, z, nthreads=None):
    x, y, z = _f32(x), _f32(y), _f32(z)
    o = np.empty_like(x)
    lib().o_expr3_f32(_p(x), _p(y), _p(z), _p(o), x.size, nthreads or threads())
    return o


def expr3_f64(x, y, z):
    x, y, z = _f32(x), _f32(y), _f32(z)
    o = np.empty(x.shape)
    lib().o_expr3_f64(_p(x), _p(y), _p(z), _p(o), x.size)
    return o


def rgb2yuv(r, g, b, nthreads=None):
    r, g, b = _f32(r), _f32(g), _f32(b)
    y, u, v = np.empty_like(r), np.empty_like(r), np.empty_like(r)
    lib().o_rgb2yuv_f32(_p(r), _p(g), _p(b), _p(y), _p(u), _p(v), r.size, nthreads or threads())
    return y, u, v


def sigmadelta(frame, bkg, var, nthreads=None):
    """One step; returns new (bkg, var, label)."""
    frame = np.ascontiguousarray(frame, dtype=np.uint8)
    bkg, var = np.array(bkg, dtype=np.uint8, copy=True), np.array(var, dtype=np.uint8, copy=True)
    label = np.empty_like(bkg)
    lib().o_sigmadelta_u8(_p(frame), _p(bkg), _p(var), _p(label), frame.size, nthreads or threads())
    return bkg, var, label


def sum_nt2(x, y=None, nthreads=None):
    x = _f32(x)
    y = None if y is None else _f32(y)
    return float(np.float32(lib().o_sum_nt2_f32(_p(x), _p(y), x.size, nthreads or threads())))


def sum_plain(x, y=None, nthreads=None):
    x = _f32(x)
    y = None if y is None else _f32(y)
    return float(np.float32(lib().o_sum_plain_f32(_p(x), _p(y), x.size, nthreads or threads())))


def globalsum(x):
    x = _f32(x)
    return float(np.float32(lib().o_globalsum_f32(_p(x), x.size)))


FOLD_OPS = {"sum": 0, "prod": 1, "max": 2, "min": 3, "mean": 4, "asum1": 5, "asum2": 6, "norm2": 7, "var": 8, "stdev": 9, "var1": 10, "stdev1": 11,
            "nbtrue": 12, "all": 13, "any": 14, "none": 15, "nansum": 16, "nanmean": 17, "meanad": 18}


def trapz_nt2(x, lo, inner, hi):
    """NT2's trapz (unit spacing) of x viewed as [lo, inner, hi] along inner."""
    x = _f32(x)
    out = np.empty(lo * hi, np.float32)
    lib().o_trapz_nt2_f32(_p(x), lo, inner, hi, _p(out))
    return out


def median(x, lo, inner, hi, ad=False):
    """NT2's median (ad: medianad) of x viewed as [lo, inner, hi] along inner."""
    x = _f32(x)
    out = np.empty(lo * hi, np.float32)
    lib().o_median_f32(_p(x), lo, inner, hi, int(ad), _p(out))
    return out


def fold_nt2(x, lo, inner, hi, op, nthreads=None):
    """NT2's in-order per-output fold of x viewed as [lo, inner, hi]:
    (float32 out[lo*hi], int64 index[lo*hi] for max/min)."""
    x = _f32(x)
    assert x.size == lo * inner * hi
    out = np.empty(lo * hi, np.float32)
    idx = np.empty(lo * hi, np.int64)
    lib().o_fold_nt2_f32(_p(x), lo, inner, hi, FOLD_OPS[op], _p(out), _p(idx), nthreads or threads())
    return out, idx


def fold_ref(x, lo, inner, hi, op, nthreads=None):
    """Reference fold: exact sums (double), sum |term| per output, max/min exact
    with NaN propagation and first-equal index."""
    x = _f32(x)
    assert x.size == lo * inner * hi
    out = np.empty(lo * hi, np.float64)
    asum = np.empty(lo * hi, np.float64)
    idx = np.empty(lo * hi, np.int64)
    lib().o_fold_ref(_p(x), lo, inner, hi, FOLD_OPS[op], _p(out), _p(asum), _p(idx), nthreads or threads())
    return out, asum, idx


SCAN_OPS = {"sum": 0, "prod": 1, "max": 2, "min": 3}


def scan_nt2(x, lo, inner, hi, op, nthreads=None):
    """NT2's in-order cumulative op of x viewed as [lo, inner, hi]."""
    x = _f32(x)
    out = np.empty(x.size, np.float32)
    lib().o_scan_nt2_f32(_p(x), lo, inner, hi, SCAN_OPS[op], _p(out), nthreads or threads())
    return out


def cumsum_exact(x, lo, inner, hi, nthreads=None):
    """Exact prefix sums (double) and the running sum of |x|."""
    x = _f32(x)
    out = np.empty(x.size, np.float64)
    ab = np.empty(x.size, np.float64)
    lib().o_cumsum_exact(_p(x), lo, inner, hi, _p(out), _p(ab), nthreads or threads())
    return out, ab


def exact_sum(x, y=None, nthreads=None):
    """Exact sum (or dot) of float data, rounded once to double; also
    returns sum |x_i| (|x_i y_i|) for the condition number."""
    x = _f32(x)
    y = None if y is None else _f32(y)
    a = ctypes.c_double()
    v = lib().o_exact_sum(_p(x), _p(y), x.size, nthreads or threads(), ctypes.byref(a))
    return v, a.value


def nt2_transform_grain(elem_size=4):
    return lib().o_nt2_transform_grain(elem_size)


# --------------------------------------------------------------- generative
# NT2's colon / linspace / logspace restated in numpy float32 (each operation
# rounded, no fusion): values at positions 0..n-1 and NT2's element counts.
#   unity colon  l + p, size (u >= l) ? size_t(u - l + 1) : 0
#                (modules/core/generative/include/nt2/core/functions/scalar/colon.hpp:24-47,
#                 details/colon.hpp unity_colon_size / unity_colon_value)
#   colon        fma(p, s, l) = p*s + l, size by tolerant_floor and fuzzy_equal
#                (scalar/colon.hpp:127-160, modules/core/fuzzy/include/nt2/fuzzy/functions/
#                 scalar/{tolerant_floor,fuzzy_equal}.hpp)
#   linspace     p == n-1 ? u : p*step + l, step = (u-l)/(n-1); n < 2 uses (u, u, 2)
#                (scalar/linspace.hpp, details/linspace.hpp)
#   logspace     exp10(p*step + lower) (scalar/logspace.hpp, details/logspace.hpp)

def _tfloor(a0):
    f = np.float32
    ct = f(3.0) * f(2.0 ** -23)
    q = f(1) - ct if a0 < 0 else f(1)
    rmax = q / (f(2) - ct)
    t1 = f(1) + f(np.floor(a0))
    t1 = (ct / q) * (-t1 if t1 < 0 else t1)
    t1 = f(np.floor(a0 + max(ct, min(rmax, t1))))
    return t1 if (a0 <= 0 or (t1 - a0) < rmax) else t1 - f(1)


def colon_size_nt2(l, s, u):
    f = np.float32
    l, s, u = f(l), f(s), f(u)
    if s == 0:
        return int(u)
    if not ((u - l) * s >= 0):
        return 0
    nelt = int(_tfloor((u - l + s) / s))
    e3 = f(3.0) * f(2.0 ** -23)
    close = lambda a, b: abs(a - b) <= e3 * max(abs(a), abs(b))  # noqa: E731
    if not close(l + f(nelt - 1) * s, u):
        if close(l + f(nelt - 2) * s, u):
            return nelt - 1
        if close(l + f(nelt) * s, u):
            return nelt + 1
    return nelt


def _pos(n, offset=0):
    return (np.arange(offset, offset + n, dtype=np.int64)).astype(np.float32)


def colon_nt2(l, s, u=None):
    f = np.float32
    if u is None:
        l, u = f(l), f(s)
        n = int(u - l + f(1)) if u >= l else 0
        return _pos(n) + l
    n = colon_size_nt2(l, s, u)
    return _pos(n) * f(s) + f(l)


def linspace_nt2(l, u, n=100):
    f = np.float32
    lo = f(u) if n < 2 else f(l)
    m = 2 if n < 2 else n
    step = (f(u) - lo) / f(m - 1)
    p = _pos(n)
    return np.where(p == f(m - 1), f(u), p * step + lo).astype(np.float32)


def logspace_nt2(l, u, n=50, regular=False):
    f = np.float32
    u = f(u)
    if not regular and u == np.uint32(0x40490fdb).view(np.float32):
        u = np.uint32(0x3efe8a6e).view(np.float32)
    lower = f(l) if n != 1 else u
    step = (u - f(l)) / f(n - 1) if n != 1 else f(0)
    return map_f32("exp10", _pos(n) * step + lower)
