"""Shared test helpers: ULP metrics and the seeded synthetic workloads.

Seeds follow the workload index: Black-Scholes plain 1000, reductions 1001,
sigma-delta / rgb2yuv 1002, batched 1003, adjoint 1004.
"""
import numpy as np

F32 = np.float32


def std_ulp(y, ref64):
    """|y - ref| in standard ulps of the float32-rounded reference (adjacent
    floats are 1 apart).  Both infinite with the same sign, or both NaN: 0."""
    y = np.asarray(y, np.float32).astype(np.float64)
    ref64 = np.asarray(ref64, np.float64)
    sp = np.spacing(np.abs(ref64.astype(np.float32))).astype(np.float64)
    with np.errstate(invalid="ignore"):
        e = np.abs(y - ref64) / sp
    same = (y == ref64) | (np.isnan(y) & np.isnan(ref64))
    return np.where(same, 0.0, e)


def nt2_ulpdist(a, b):
    """NT2's ulpdist for float (frexp mantissa difference / Eps): half of the
    standard ulp distance.  modules/boost/simd/base/include/boost/simd/ieee/
    functions/scalar/ulpdist.hpp:56-80; modules/test/unit/src/ulp.cpp:18-32."""
    a, b = np.float32(a), np.float32(b)
    if a == b or (np.isnan(a) and np.isnan(b)):
        return 0.0
    if not (np.isfinite(a) and np.isfinite(b)):
        return np.inf
    m1, e1 = np.frexp(a)
    m2, e2 = np.frexp(b)
    expo = -max(e1, e2)
    if e1 == e2:
        e = abs(np.float32(m1) - np.float32(m2))
    else:
        e = abs(np.float32(np.ldexp(a, expo)) - np.float32(np.ldexp(b, expo)))
    return float(e) / float(np.finfo(np.float32).eps)


def conditioned_ulp(y, ref64, scale64):
    """|y - ref| in ulps of the largest cancelling term (Black-Scholes call =
    S*N(d1) - K e^-rT N(d2): the terms, not the difference, set the scale)."""
    sp = np.spacing(np.abs(np.asarray(scale64, np.float64)).astype(np.float32)).astype(np.float64)
    return np.abs(np.asarray(y, np.float64) - ref64) / sp


# Stated accuracy of the fast-policy Black-Scholes call/put against FP64, in
# conditioned ulps (error over the ulp of the larger cancelling term): the
# bound the GPU tests assert (measured maxima: 12.3 over the 5.7e7 options of
# the batched mix, about 10.8 over the 2^20 bench options; NT2's own float
# evaluation of the same options: 300-400).
BS_FAST_MAX, BS_FAST_P999, BS_FAST_MEAN, BS_FAST_CORE = 14.0, 6.0, 1.1, 8.0


def bs_inputs(n, seed=1000, sigma_table=False):
    rng = np.random.default_rng(seed)
    S = rng.uniform(5, 30, n).astype(F32)
    K = rng.uniform(1, 100, n).astype(F32)
    T = rng.uniform(0.25, 10, n).astype(F32)
    if sigma_table:
        return S, K, T, rng.uniform(0.05, 0.8, n).astype(F32)
    return S, K, T


def reduction_well(n, seed=1001):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(n, dtype=F32), rng.standard_normal(n, dtype=F32)


def reduction_ill(n, seed=1001, target_cond=1e10):
    """Exact-cancelling pairs (+a, -a), a = +-2^e with e ~ U{-40..40}, at
    random positions, over an N(0, 1e-3) residue; pairs are added until
    sum|x| / |sum x| reaches the target (the realised value is returned)."""
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal(n) * 1e-3).astype(F32)
    total = float(np.sum(x.astype(np.float64)))
    absum = float(np.sum(np.abs(x.astype(np.float64))))
    goal = target_cond * abs(total)
    pos = rng.permutation(n)
    k = 0
    while absum < goal and 2 * k + 1 < n:
        e = int(rng.integers(-40, 41))
        a = np.float32(np.ldexp(1.0, e)) * (1 if rng.random() < 0.5 else -1)
        if absum + 2 * abs(float(a)) > 2 * goal:  # keep the realised value near the target
            if abs(float(a)) > goal:
                continue
        i, j = pos[2 * k], pos[2 * k + 1]
        total -= float(x[i]) + float(x[j])
        absum -= abs(float(x[i])) + abs(float(x[j]))
        x[i], x[j] = a, -a
        absum += 2 * abs(float(a))
        k += 1
    return x


def reduction_ill_dot(n, seed=1001, target_cond=1e10):
    """dot(x, y) with condition number sum|x*y| / |sum x*y| near target_cond:
    over an x ~ N(0,1), y ~ N(0,1e-3) residue, pairs of positions carry
    products that cancel exactly, (a, b) and (-a, b) with a = +-m 2^e,
    b = m' 2^e' (m, m' ~ U[1,2), e, e' ~ U{-20..20}).  Float products are
    exact in FP64, so the exact dot is the residue's."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(n).astype(F32)
    y = (rng.standard_normal(n) * 1e-3).astype(F32)
    p = x.astype(np.float64) * y.astype(np.float64)
    total = float(np.sum(p))
    absum = float(np.sum(np.abs(p)))
    goal = target_cond * abs(total)
    pos = rng.permutation(n)
    k = 0
    while absum < goal and 2 * k + 1 < n:
        a = np.float32(np.ldexp(rng.uniform(1, 2), int(rng.integers(-20, 21)))) * (1 if rng.random() < 0.5 else -1)
        b = np.float32(np.ldexp(rng.uniform(1, 2), int(rng.integers(-20, 21))))
        mag = abs(float(a) * float(b))
        if absum + 2 * mag > 2 * goal and mag > goal:
            continue
        i, j = pos[2 * k], pos[2 * k + 1]
        total -= float(p[i]) + float(p[j])
        absum -= abs(float(p[i])) + abs(float(p[j]))
        x[i], y[i], x[j], y[j] = a, b, -a, b
        absum += 2 * mag
        k += 1
    return x, y


def sigmadelta_frames(h=1080, w=1920, frames=64, seed=1002, square=200, step=8):
    """uint8 frames ~ U[0,255] with a bright square moving `step` px per frame."""
    rng = np.random.default_rng(seed)
    f = rng.integers(0, 256, size=(frames, h, w), dtype=np.uint8)
    for k in range(frames):
        x0 = (k * step) % w
        cols = (np.arange(square) + x0) % w
        y0 = (h - square) // 2
        f[k, y0:y0 + square][:, cols] = 255
    return f


def rgb_planes(n, seed=1002):
    rng = np.random.default_rng(seed)
    return tuple(rng.uniform(0, 1, n).astype(F32) for _ in range(3))


def batched_sizes(count=4096, lo=1024, hi=4194304, seed=1003):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), count)).astype(np.int64)
    exprs = rng.integers(0, 3, count)
    return sizes, exprs


# ------------------------------------------------------------ reverse mode --
# FP64 forward-mode dual numbers: the reference the program-level VJP is
# checked against (a method independent of the kernel's reverse sweep).  A
# Dual carries its value, the tangents along each input direction, and the
# absolute tangents -- the sum over the expression's paths of |product of the
# local partials| -- which are the gradient's term scale: the size of the terms
# its chain-rule sum adds, the gradient's own magnitude except where they
# cancel.
class Dual:
    __slots__ = ("v", "t", "a")

    def __init__(self, v, t, a):
        self.v, self.t, self.a = v, t, a

    @staticmethod
    def var(x, i, k):
        x = np.asarray(x, np.float64)
        t = np.zeros((k,) + x.shape)
        t[i] = 1.0
        return Dual(x, t, t.copy())

    @staticmethod
    def lift(c, like):
        if isinstance(c, Dual):
            return c
        return Dual(np.broadcast_to(np.float64(c), like.v.shape), np.zeros_like(like.t), np.zeros_like(like.a))

    def _un(self, v, d):
        return Dual(v, d * self.t, np.abs(d) * self.a)

    def __add__(self, o):
        o = Dual.lift(o, self)
        return Dual(self.v + o.v, self.t + o.t, self.a + o.a)

    __radd__ = __add__

    def __sub__(self, o):
        o = Dual.lift(o, self)
        return Dual(self.v - o.v, self.t - o.t, self.a + o.a)

    def __rsub__(self, o):
        return Dual.lift(o, self) - self

    def __neg__(self):
        return Dual(-self.v, -self.t, self.a)

    def __mul__(self, o):
        o = Dual.lift(o, self)
        return Dual(self.v * o.v, self.t * o.v + self.v * o.t, self.a * np.abs(o.v) + np.abs(self.v) * o.a)

    __rmul__ = __mul__

    def __truediv__(self, o):
        o = Dual.lift(o, self)
        q = self.v / o.v
        return Dual(q, (self.t - q * o.t) / o.v, self.a / np.abs(o.v) + np.abs(q / o.v) * o.a)

    def __rtruediv__(self, o):
        return Dual.lift(o, self) / self


def d_sqrt(x):
    r = np.sqrt(x.v)
    return x._un(r, 0.5 / r)


def d_log(x):
    return x._un(np.log(x.v), 1.0 / x.v)


def d_log1p(x):
    return x._un(np.log1p(x.v), 1.0 / (1.0 + x.v))


def d_exp(x):
    e = np.exp(x.v)
    return x._un(e, e)


def d_abs(x):
    return x._un(np.abs(x.v), np.sign(x.v))


def d_sqr(x):
    return x * x


def d_fma(a, b, c):
    return a * b + c


def d_fnms(a, b, c):
    return c - a * b


def d_normcdf(x):
    from scipy.special import ndtr
    return x._un(ndtr(x.v), np.exp(-0.5 * x.v * x.v) / np.sqrt(2 * np.pi))


# NT2's fastnormcdf (Abramowitz-Stegun 26.2.17 with NT2's float coefficients)
# and its exact derivative, in FP64.
_AS_P = float(np.float32(0.2316419))
_AS_B = [float(np.uint32(u).view(np.float32)) for u in (0x3ea385fa, 0xbeb68f87, 0x3fe40778, 0xbfe91eea, 0x3faa466f)]


def fastnormcdf64(x):
    x = np.asarray(x, np.float64)
    b1, b2, b3, b4, b5 = _AS_B
    l = np.abs(x)
    k = 1.0 / (1.0 + _AS_P * l)
    q = b1 + k * (b2 + k * (b3 + k * (b4 + k * b5)))
    dq = b2 + k * (2 * b3 + k * (3 * b4 + k * 4 * b5))
    e = np.exp(-0.5 * l * l) / np.sqrt(2 * np.pi)
    w = e * k * q
    f = np.where(x > 0, 1.0 - w, w)
    df = e * k * (l * q + _AS_P * k * (q + k * dq))
    return f, df


def d_fastnormcdf(x):
    f, df = fastnormcdf64(x.v)
    return x._un(f, df)


def bs_demo_dual(S, X, T, r, v):
    """The NT2 demo's Black-Scholes expression (demo/blackscholes/nt2/
    blackandscholes_nt2.cpp:55-59), operation for operation, on Duals."""
    da = d_sqrt(T)
    d1 = d_log(S / X) + (d_fma(d_sqr(v), 0.5, r) * T) / (v * da)
    d2 = d_fnms(v, da, d1)
    return d_fnms(X * d_exp(-r * T), d_fastnormcdf(d2), S * d_fastnormcdf(d1))


def bs_textbook_dual(S, K, T, sig, r):
    """Textbook Black-Scholes call and put (normcdf), operation for operation
    as the tests write the expression, on Duals."""
    sq = d_sqrt(T)
    d1 = (d_log(S / K) + d_fma(d_sqr(sig), 0.5, r) * T) / (sig * sq)
    d2 = d_fnms(sig, sq, d1)
    e = K * d_exp(-r * T)
    return d_fnms(e, d_normcdf(d2), S * d_normcdf(d1)), d_fnms(S, d_normcdf(-d1), e * d_normcdf(-d2))
