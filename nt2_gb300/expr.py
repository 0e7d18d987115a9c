"""A Python mirror of NT2's expression surface over device tables.

``Table`` wraps a CUDA tensor; arithmetic operators and the NT2 functor names
(exp, exp2, exp10, expm1, log, log2, log10, log1p, sin, cos, tan, cot, sec, csc, sinpi, cospi,
tanpi, proper_tanpi, cotpi, secpi, cscpi, sind, cosd, tand, cotd, secd, cscd, sinc, sincpi, pow,
sinh, cosh, tanh, coth, sech, csch, sinhc, asinh, acosh, atanh, asech, acsch, acoth,
asin, acos, atan, acot, asec, acsc, asind, acosd, atand, acotd, asecd, acscd,
asinpi, acospi, atanpi, atan2, atan2d, indeg, inrad, cbrt, hypot,
erfc, normcdf, fastnormcdf, sqrt, sqr, abs, rec, fma, fnms, min, max, if_else,
selinc, seldec, if_zero_else_one, adds) build an expression
tree; ``assign(outs, exprs)`` is ``tie(outs...) = tie(exprs...)``: it lowers
the trees to the SSA program of nt2g.h, compiles it once (cached by program
text) and evaluates it through ``nt2g_eval`` -- the same path the C++ table
layer takes (nt2_gb300/include/nt2/table.hpp).

Mirrors: run_assign -> transform lowering, modules/core/base/include/nt2/dsl/
functions/elementwise/run.hpp:21-36; tie, modules/core/container/table/include/
nt2/core/functions/expr/tie.hpp:40-121; partial transform ranges,
modules/core/container/table/include/nt2/core/functions/expr/transform.hpp:40-60.
"""
import ctypes

from . import lib


class Node:
    __slots__ = ("op", "args", "dtype", "imm", "table", "numel")

    def __init__(self, op, args=(), dtype=lib.F32, imm=0.0, table=None, numel=None):
        self.op, self.args, self.dtype, self.imm, self.table = op, tuple(args), dtype, imm, table
        self.numel = numel  # element count of a generative (INDEX) leaf

    # arithmetic
    def __add__(self, o): return _bin("ADD", self, o)
    def __radd__(self, o): return _bin("ADD", o, self)
    def __sub__(self, o): return _bin("SUB", self, o)
    def __rsub__(self, o): return _bin("SUB", o, self)
    def __mul__(self, o): return _bin("MUL", self, o)
    def __rmul__(self, o): return _bin("MUL", o, self)
    def __truediv__(self, o): return _bin("DIV", self, o)
    def __rtruediv__(self, o): return _bin("DIV", o, self)
    def __neg__(self): return Node("NEG", (self,), self.dtype)
    # comparisons produce logicals
    def __lt__(self, o): return _bin("LT", self, o)
    def __gt__(self, o): return _bin("GT", self, o)
    def __le__(self, o): return _bin("LE", self, o)
    def __ge__(self, o): return _bin("GE", self, o)
    def ne(self, o): return _bin("NE", self, o)
    def eq(self, o): return _bin("EQ", self, o)
    __hash__ = object.__hash__


# Leaves are plain Nodes (not subclasses): with a subclass on the right,
# Python would try its reflected comparison first and turn d < var into
# var > d, which computes the same but no longer has the expression's shape.
def Table(tensor):
    """A device table leaf (CUDA tensor, float32 or uint8)."""
    import torch
    if tensor.dtype not in (torch.uint8, torch.float32):
        raise TypeError(f"tables hold float32 or uint8, not {tensor.dtype}")
    return Node("LOAD", (), lib.U8 if tensor.dtype == torch.uint8 else lib.F32, table=tensor)


def Scalar(value, dtype=lib.F32):
    """A run-time scalar argument (a SCALAR slot, not baked into the program)."""
    return Node("SCALAR", (), dtype, imm=float(value))


def _wrap(x, dtype):
    if isinstance(x, Node):
        return x
    return Node("CONST", (), dtype, imm=float(x))


def _bin(op, a, b):
    dt = a.dtype if isinstance(a, Node) else b.dtype
    return Node(op, (_wrap(a, dt), _wrap(b, dt)), dt)


def _un(op):
    return lambda a: Node(op, (a,), a.dtype)


exp, log, log1p, erfc = _un("EXP"), _un("LOG"), _un("LOG1P"), _un("ERFC")
normcdf, fastnormcdf, sqrt, rec = _un("NORMCDF"), _un("FASTNORMCDF"), _un("SQRT"), _un("REC")
abs_ = _un("ABS")
exp2, exp10, expm1 = _un("EXP2"), _un("EXP10"), _un("EXPM1")
log2, log10 = _un("LOG2"), _un("LOG10")
sin, cos, tan, sinpi, cospi = _un("SIN"), _un("COS"), _un("TAN"), _un("SINPI"), _un("COSPI")
sinh, cosh, tanh = _un("SINH"), _un("COSH"), _un("TANH")
asin, acos, atan = _un("ASIN"), _un("ACOS"), _un("ATAN")
asinh, acosh, atanh = _un("ASINH"), _un("ACOSH"), _un("ATANH")
cbrt = _un("CBRT")
cot, sec, csc = _un("COT"), _un("SEC"), _un("CSC")
sind, cosd, tand = _un("SIND"), _un("COSD"), _un("TAND")
tanpi = _un("TANPI")
proper_tanpi = _un("PROPER_TANPI")
cotpi = _un("COTPI")
cotd = _un("COTD")
secpi = _un("SECPI")
cscpi = _un("CSCPI")
secd = _un("SECD")
cscd = _un("CSCD")
sinc = _un("SINC")
sincpi = _un("SINCPI")
acotd = _un("ACOTD")
asec = _un("ASEC")
coth = _un("COTH")
sinhc = _un("SINHC")
acsc = _un("ACSC")
asech = _un("ASECH")
acoth = _un("ACOTH")
acsch = _un("ACSCH")
erf = _un("ERF")
erfcx = _un("ERFCX")
expx2 = _un("EXPX2")
gamma = _un("GAMMA")
gammaln = _un("GAMMALN")
digamma = _un("DIGAMMA")
signgam = _un("SIGNGAM")
dawson = _un("DAWSON")
spence = _un("SPENCE")
stirling = _un("STIRLING")


# NT2's beta and betaln, built as NT2 writes them (EUL/scalar/beta.hpp:
# sign*exp(gammaln(a0)+gammaln(a1)-gammaln(y)) with y = a0+a1 and sign =
# signgam(a0)*signgam(a1)*signgam(y); EUL/simd/common/betaln.hpp:
# gammaln(a0)+gammaln(a1)-gammaln(a0+a1))
def beta(a, b):
    y = a + b
    return (signgam(a) * signgam(b)) * signgam(y) * exp(gammaln(a) + gammaln(b) - gammaln(y))


def betaln(a, b):
    return gammaln(a) + gammaln(b) - gammaln(a + b)
erfinv = _un("ERFINV")
erfcinv = _un("ERFCINV")
floor = _un("FLOOR")
ceil = _un("CEIL")
trunc = _un("TRUNC")
round = _un("ROUND")
round2even = _un("ROUND2EVEN")
frac = _un("FRAC")
sign = _un("SIGN")
signnz = _un("SIGNNZ")
fix = trunc


# predicates (boost/simd/predicates/functions): logical results for if_else
def _pred(op):
    return lambda a: Node(op, (a,), a.dtype)


is_nan, is_inf, is_finite = _pred("IS_NAN"), _pred("IS_INF"), _pred("IS_FINITE")
is_eqz, is_nez, is_ltz, is_gtz = _pred("IS_EQZ"), _pred("IS_NEZ"), _pred("IS_LTZ"), _pred("IS_GTZ")


def copysign(a, b): return _bin("COPYSIGN", a, b)


def mod(a, b):
    """NT2's mod: a - floor(a/b) b, a where b == 0."""
    return _bin("MOD", a, b)


def pow2(a, b=None):
    """NT2's pow2: a * 2^trunc(b) by fast_ldexp (pow2(x) = 2^trunc(x))."""
    return _bin("POW2", 1.0, a) if b is None else _bin("POW2", a, b)


def rem(a, b):
    """NT2's rem: a - b itrunc(a/b) (the quotient through a saturating int32), a where b == 0."""
    return _bin("REM", a, b)


# oneplus, oneminus, minusone, sqr_abs, dist, average: boost/simd/arithmetic/
# functions/generic/{oneplus,oneminus,minusone,sqr_abs,average}.hpp, scalar/dist.hpp
def oneplus(a): return a + 1.0
def oneminus(a): return 1.0 - a
def minusone(a): return a - 1.0


# the saturating and increment forms of boost.simd as they are for floats
# (boost/simd/arithmetic/functions/{generic/inc,generic/dec,generic/abss,
# scalar/negs,scalar/sqrs,generic/conj}.hpp): a + 1, a - 1, abs, -a, sqr, a
def inc(a): return a + 1.0
def dec(a): return a - 1.0
def abss(a): return abs_(a)
def negs(a): return -a
def sqrs(a): return sqr(a)
def conj(a): return a
def sqr_abs(a): return sqr(a)
def dist(a, b): return abs_(a - b)
def average(a, b): return fma(a, 0.5, b * 0.5)
exprecneg = _un("EXPRECNEG")
exprecnegc = _un("EXPRECNEGC")
sqrt1pm1 = _un("SQRT1PM1")


# NT2's generic compositions, built as the same programs of the functors above,
# operation for operation (hyperbolic/functions/generic/{sech,csch}.hpp;
# trigonometric/functions/generic/{acot,indeg,inrad,asind,acosd,atand,asecd,
# acscd,atan2d,asinpi,acospi,atanpi}.hpp)
def _bits_f32(u):
    import struct
    return struct.unpack("<f", struct.pack("<I", u))[0]


_RADINDEG, _RADINDEGR = _bits_f32(0x42652ee1), _bits_f32(0xb53387c1)
_DEGINRAD, _INVPI = _bits_f32(0x3c8efa35), _bits_f32(0x3ea2f983)


def sech(a): return rec(cosh(a))
def csch(a): return rec(sinh(a))
def acot(a): return atan(rec(a))
def indeg(a): return a * _RADINDEG - a * _RADINDEGR
def inrad(a): return a * _DEGINRAD
def asind(a): return indeg(asin(a))
def acosd(a): return indeg(acos(a))
def atand(a): return indeg(atan(a))
def asecd(a): return indeg(asec(a))
def acscd(a): return indeg(acsc(a))
def atan2d(a, b): return indeg(atan2(a, b))
def asinpi(a): return _INVPI * asin(a)
def acospi(a): return _INVPI * acos(a)
def atanpi(a): return _INVPI * atan(a)


# Distribution functions of NT2's statistics module as NT2 composes them
# (modules/core/statistics/include/nt2/statistics/functions/generic/*.hpp), every operation in NT2's order:
# if_zero_else(c, x) = c ? 0 : x, if_allbits_else(c, x) = c ? NaN : x, and
# is_not_greater(a, b) = !(a > b).  Parameters are numbers or expressions.
_INVSQRT_2PI, _SQRT_2, _SQRT_2O_2 = _bits_f32(0x3ecc422a), _bits_f32(0x3fb504f3), _bits_f32(0x3f3504f3)
_NAN = float("nan")


def _is_negative(a):  # the sign bit (boost.simd is_negative: -0 included)
    return copysign(1.0, a) < 0.0


def is_lez(a):
    """boost.simd is_lez: a <= 0 (false for NaN)."""
    return a <= 0.0


def _p(v):
    """A parameter as a node: numbers become run-time float scalars, so that
    every operation on them is NT2's float operation on the device."""
    return v if v is None or isinstance(v, Node) else Scalar(v)


def normpdf(x, m=None, s=None):
    """normpdf.hpp: exp(-1/2 sqr((x - m) rec(s))) / sqrt(2 pi) rec(s)."""
    m, s = _p(m), _p(s)
    if s is not None:
        inv = rec(s)
        return exp(-0.5 * sqr((x - m) * inv)) * _INVSQRT_2PI * inv
    return exp(-0.5 * sqr(x if m is None else x - m)) * _INVSQRT_2PI


def norminv(p, m=None, s=None):
    """norminv.hpp: -sqrt(2) erfcinv(2 p), then + m or fma(., s, m)."""
    m, s = _p(m), _p(s)
    z = -_SQRT_2 * erfcinv(2.0 * p)
    if s is not None:
        return fma(z, s, m)
    return z if m is None else z + m


def expcdf(x, mu=None):
    """expcdf.hpp: -expm1(-if_zero_else(is_ltz(x), x)) of x (or x / mu)."""
    mu = _p(mu)
    if mu is not None:
        x = x / mu
    return -expm1(-if_else(is_ltz(x), 0.0, x))


def exppdf(x, lam=None):
    """exppdf.hpp: if_zero_else(is_ltz(x), exp(-x)) or lam exp(-x lam)."""
    lam = _p(lam)
    return if_else(is_ltz(x), 0.0, exp(-x) if lam is None else lam * exp(-x * lam))


def expinv(p, mu=None):
    """expinv.hpp: if_allbits_else(is_ltz(p), -log1p(-p)), times mu."""
    mu = _p(mu)
    r = if_else(is_ltz(p), _NAN, -log1p(-p))
    return r if mu is None else mu * r


def logncdf(x, m=None, s=None):
    """logncdf.hpp: erfc(-sqrt(1/2) log(x)) / 2, log(x) -> (m - log(x)) [/ s]; x <= 0 read as 0."""
    m, s = _p(m), _p(s)
    lx = log(if_else(is_lez(x), 0.0, x))
    if m is None:
        return 0.5 * erfc(-_SQRT_2O_2 * lx)
    t = m - lx
    return 0.5 * erfc(_SQRT_2O_2 * (t if s is None else t / s))


def lognpdf(x, m=None, s=None):
    """lognpdf.hpp: normpdf(log(x)[, m[, s]]) / x, x <= 0 read as +inf."""
    m, s = _p(m), _p(s)
    xx = if_else(is_lez(x), float("inf"), x)
    return normpdf(log(xx), m, s) / xx


def logninv(p, m=None, s=None):
    """logninv.hpp: exp(-sqrt(2) [s] erfcinv(2 p) [+ m])."""
    m, s = _p(m), _p(s)
    c = -_SQRT_2 if s is None else -_SQRT_2 * s
    z = c * erfcinv(2.0 * p)
    return exp(z if m is None else z + m)


def unifcdf(x, a=None, b=None):
    """unifcdf.hpp: x clamped to [0, 1]; with [a, b]: NaN for b <= a, else 0 below a,
    (x - a) / (b - a) up to b, 1 above."""
    a, b = _p(a), _p(b)
    if a is None:
        return if_else(is_ltz(x), 0.0, if_else(x > 1.0, 1.0, x))
    z = b - a
    return if_else(is_lez(z), _NAN, if_else(x < a, 0.0, if_else(x > b, 1.0, (x - a) / z)))


def unifpdf(x, a=None, b=None):
    """unifpdf.hpp: 1 on [0, 1] (not at -0), NaN for NaN; with [a, b]: rec(b - a) inside,
    0 outside, NaN for b <= a or a NaN x."""
    a, b = _p(a), _p(b)
    if a is None:
        return if_else(is_nan(x), x, if_else(x <= 1.0, if_else(_is_negative(x), 0.0, 1.0), 0.0))
    z = b - a
    return if_else(is_lez(z), _NAN, if_else(is_nan(x), _NAN, if_else(x < a, 0.0, if_else(x > b, 0.0, rec(z)))))


def unifinv(p, a=None, b=None):
    """unifinv.hpp: p on [0, 1], else NaN; with [a, b] NT2's fma(p, if_allbits_else(p > b or
    p < a, b - a), a) as written."""
    a, b = _p(a), _p(b)
    if a is None:
        return if_else(p < 0.0, _NAN, if_else(p <= 1.0, p, _NAN))
    return fma(p, if_else(p > b, _NAN, if_else(p < a, _NAN, b - a)), a)


def caucdf(x, m=None, s=None):
    """caucdf.hpp: 1/2 + atanpi(x), x -> x - m or (x - m) / s."""
    m, s = _p(m), _p(s)
    if m is not None:
        x = x - m if s is None else (x - m) / s
    return 0.5 + atanpi(x)


def cauinv(p, m=None, s=None):
    """cauinv.hpp: proper_tanpi(p - 1/2), then + m or fma(., s, m)."""
    m, s = _p(m), _p(s)
    z = proper_tanpi(p - 0.5)
    if s is not None:
        return fma(z, s, m)
    return z if m is None else z + m


def caupdf(x, m=None, s=None):
    """caupdf.hpp: rec(oneplus(sqr(x))) / pi (x -> x - m), or (s / pi) / (sqr(s) + sqr(x - m))."""
    m, s = _p(m), _p(s)
    if s is None:
        return rec(1.0 + sqr(x if m is None else x - m)) * _INVPI
    return (s * _INVPI) / (sqr(s) + sqr(x - m))


def evcdf(x, m=None, s=None):
    """evcdf.hpp: -expm1(-exp(x)), x -> x - m or (x - m) / s."""
    m, s = _p(m), _p(s)
    if m is not None:
        x = x - m if s is None else (x - m) / s
    return -expm1(-exp(x))


def evpdf(x, m=None, s=None):
    """evpdf.hpp: t = exp(x'), t * exp(-t) [* rec(s)], 0 at x = +inf."""
    m, s = _p(m), _p(s)
    if s is not None:
        inv = rec(s)
        t = exp((x - m) * inv)
        t = t * (exp(-t) * inv)
    else:
        t = exp(x if m is None else x - m)
        t = t * exp(-t)
    return if_else(x.eq(float("inf")), 0.0, t)


def evinv(p, m=None, s=None):
    """evinv.hpp: log(-log1p(-p)) [* s] [+ m]."""
    m, s = _p(m), _p(s)
    z = log(-log1p(-p))
    if s is not None:
        z = z * s
    return z if m is None else z + m


# logspace_add, logspace_sub (exponential/functions/scalar/logspace_add.hpp,
# logspace_sub.hpp) in NT2's forms; NT2's max(a, b) is a > b ? a : b.  The
# real* functors are NT2's assertion-only aliases of sqrt, log and pow.
def logspace_add(a, b):
    t = -abs_(a - b)
    return if_else(_bin("NE", t, t), a + b, max_(a, b) + log1p(exp(t)))


def logspace_sub(a, b):
    d = b - a
    return a + if_else(d > -_bits_f32(0x3f317218), log(-expm1(d)), log1p(-exp(d)))


realsqrt, reallog = sqrt, log


def realpow(a, b): return pow(a, b)

# Functors applied to plain numbers evaluate at once in float32 with NT2's
# scalar semantics (each step rounded, no fusion), as NT2's scalar overloads
# do in C++ before an expression is built.


def _f32(x):
    import numpy as np
    return np.float32(x)


def sqr(a):
    if isinstance(a, Node):
        return Node("SQR", (a,), a.dtype)
    return float(_f32(a) * _f32(a))


def fma(a, b, c):
    if not any(isinstance(x, Node) for x in (a, b, c)):
        return float(_f32(_f32(a) * _f32(b)) + _f32(c))
    dt = next(x.dtype for x in (a, b, c) if isinstance(x, Node))
    return Node("FMA", tuple(_wrap(x, dt) for x in (a, b, c)), dt)


def fnms(a, b, c):
    """c - a*b"""
    if not any(isinstance(x, Node) for x in (a, b, c)):
        return float(_f32(c) - _f32(_f32(a) * _f32(b)))
    dt = next(x.dtype for x in (a, b, c) if isinstance(x, Node))
    return Node("FNMS", tuple(_wrap(x, dt) for x in (a, b, c)), dt)


def pow(a, b):
    """a^b with NT2's semantics (NaN for a < 0 and non-integer b, pow(0, b) = (b == 0))."""
    if not any(isinstance(x, Node) for x in (a, b)):
        raise TypeError("pow of two numbers: use Python's ** (NT2's scalar pow is not mirrored here)")
    return _bin("POW", a, b)


def hypot(a, b):
    """sqrt(a^2 + b^2) without undue overflow (NT2's scaled form)."""
    return _bin("HYPOT", a, b)


def nthroot(x, n):
    """NT2's real n-th root of x (n truncated toward zero; NaN for x < 0 and even n)."""
    return _bin("NTHROOT", x, n)


def expni(n, x):
    """NT2's exponential integral E_n(x) (n truncated toward zero)."""
    return _bin("EXPNI", n, x)


def gammainc(x, a):
    """NT2's regularised lower incomplete gamma function P(a, x), evaluated in double."""
    return _bin("GAMMAINC", x, a)


def gammaincinv(p, a):
    """NT2's gammaincinv(p, a): the x with P(a, x) = p (+inf for p = 1), in double."""
    return _bin("GAMMAINCINV", p, a)


def atan2(a, b):
    """atan2(a, b) with NT2's semantics (atan2(+-0, b < 0) = pi)."""
    return _bin("ATAN2", a, b)


def min_(a, b): return _bin("MIN", a, b)
def max_(a, b): return _bin("MAX", a, b)
def adds(a, b): return _bin("ADDS", a, b)


def if_else(c, a, b):
    dt = a.dtype if isinstance(a, Node) else b.dtype if isinstance(b, Node) else lib.F32
    return Node("IF_ELSE", (c, _wrap(a, dt), _wrap(b, dt)), dt)


# boost.simd's NaN-ignoring and magnitude selects, minmod, negate, fms and fnma
# as their scalar float definitions compose them
# (boost/simd/ieee/functions/scalar/{maxnum,minnum,maxmag,minmag,negate}.hpp,
# boost/simd/arithmetic/functions/{scalar/minmod,generic/fms,generic/fnma}.hpp)
def maxnum(a, b):
    """is_nan(a) ? b : max(b, a)."""
    a, b = _p(a), _p(b)
    return if_else(is_nan(a), b, max_(b, a))


def minnum(a, b):
    """is_nan(a) ? b : min(b, a)."""
    a, b = _p(a), _p(b)
    return if_else(is_nan(a), b, min_(b, a))


def maxmag(a, b):
    """|a| > |b| ? a : |b| > |a| ? b : max(a, b)."""
    a, b = _p(a), _p(b)
    return if_else(abs_(a) > abs_(b), a, if_else(abs_(b) > abs_(a), b, max_(a, b)))


def minmag(a, b):
    """|a| < |b| ? a : |b| < |a| ? b : min(a, b)."""
    a, b = _p(a), _p(b)
    return if_else(abs_(a) < abs_(b), a, if_else(abs_(b) < abs_(a), b, min_(a, b)))


def minmod(a, b):
    """is_nltz(a*b) ? min(a, b) : 0."""
    a, b = _p(a), _p(b)
    return if_else(a * b < 0.0, 0.0, min_(a, b))


def negate(a, b):
    """a * sign(b)."""
    return _p(a) * sign(_p(b))


def fms(a, b, c):
    """a*b - c (a product and a difference, as NT2 writes it)."""
    return _p(a) * _p(b) - _p(c)


def fnma(a, b, c):
    """-c - a*b."""
    return -_p(c) - _p(a) * _p(b)


# boost.simd's rounded quotients for floats (boost/simd/arithmetic/functions/
# scalar/{divfloor,divceil,divfix,divround,divround2even}.hpp): the rounding
# of the correctly rounded a/b (both policies divide correctly rounded)
def divfloor(a, b): return floor(_p(a) / _p(b))
def divceil(a, b): return ceil(_p(a) / _p(b))
def divfix(a, b): return trunc(_p(a) / _p(b))
def divround(a, b): return round(_p(a) / _p(b))
def divround2even(a, b): return round2even(_p(a) / _p(b))


def selinc(c, a): return Node("SELINC", (c, a), a.dtype)
def seldec(c, a): return Node("SELDEC", (c, a), a.dtype)
def if_zero_else_one(c, dtype): return Node("IF_ZERO_ELSE_ONE", (c,), dtype)


# ------------------------------------------------------------------ generative
# colon / linspace / logspace over the element position p (NT2's
# enumerate<T>(p), the INDEX leaf); sizes and steps in float32 with every step
# rounded, as NT2 computes them (modules/core/generative/include/nt2/core/
# functions/scalar/{colon,linspace,logspace}.hpp, details/*.hpp,
# modules/core/fuzzy/include/nt2/fuzzy/functions/scalar/tolerant_floor.hpp).

def _index(n):
    return Node("INDEX", (), lib.F32, numel=int(n))


def _generative_sizes(e, seen=None):
    seen = set() if seen is None else seen
    if id(e) in seen or not isinstance(e, Node):
        return []
    seen.add(id(e))
    out = [e.numel] if e.op in ("INDEX", "CONST") and e.numel is not None else []
    for a in e.args:
        out += _generative_sizes(a, seen)
    return out



def _tolerant_floor(a0):
    import numpy as np
    f = np.float32
    ct = f(3) * f(np.finfo(np.float32).eps)
    q = f(1) - ct if a0 < 0 else f(1)
    rmax = q / (f(2) - ct)
    t1 = f(1) + np.floor(a0)
    t1 = (ct / q) * (-t1 if t1 < 0 else t1)
    lo = rmax if rmax < t1 else t1
    t1 = np.floor(a0 + (ct if ct > lo else lo))
    return t1 if (a0 <= 0 or (t1 - a0) < rmax) else t1 - f(1)


def _check_generative_sizes(exprs, count):
    """NT2 assigns an expression only to a table of its own size: generative
    leaves must have as many elements as the full assignment."""
    sizes = {m for e in exprs for m in _generative_sizes(e)}
    if sizes and sizes != {count}:
        raise ValueError(f"generative operands of {sorted(sizes)} elements assigned to {count}")


def ones(*size):
    """A constant table of ones: ones(n) is n x n, ones(a, b, ...) has a*b*... elements."""
    import math
    return Node("CONST", (), lib.F32, imm=1.0, numel=size[0] * size[0] if len(size) == 1 else math.prod(size))


def zeros(*size):
    import math
    return Node("CONST", (), lib.F32, imm=0.0, numel=size[0] * size[0] if len(size) == 1 else math.prod(size))


def colon_count(l, s, u):
    """NT2's element count of colon(l, s, u) on floats."""
    import numpy as np
    f = np.float32
    l, s, u = f(l), f(s), f(u)
    if not s:
        return int(u)
    if not ((u - l) * s >= 0):
        return 0
    nelt = int(_tolerant_floor((u - l + s) / s))
    eps3 = f(3) * f(np.finfo(np.float32).eps)

    def feq(a, b):
        return abs(a - b) <= eps3 * max(abs(a), abs(b))
    if not feq(l + f(nelt - 1) * s, u):
        if feq(l + f(nelt - 2) * s, u):
            return nelt - 1
        if feq(l + f(nelt) * s, u):
            return nelt + 1
    return nelt


def colon(l, s_or_u, u=None):
    """colon(l, u) = l + p over u-l+1 elements; colon(l, s, u) = fma(p, s, l)."""
    import numpy as np
    if u is None:
        lf, uf = np.float32(l), np.float32(s_or_u)
        n = int(uf - lf + np.float32(1)) if uf >= lf else 0
        return Node("ADD", (_index(n), _wrap(float(lf), lib.F32)), lib.F32)
    n = colon_count(l, s_or_u, u)
    return Node("FMA", (_index(n), _wrap(float(np.float32(s_or_u)), lib.F32), _wrap(float(np.float32(l)), lib.F32)),
                lib.F32)


def linspace(l, u, n=100):
    """n points from l to u: p == n-1 ? u : fma(p, (u-l)/(n-1), l)."""
    import numpy as np
    f = np.float32
    lo = f(u) if n < 2 else f(l)
    m = 2 if n < 2 else n
    step = (f(u) - lo) / f(m - 1)
    p = _index(n)
    last = Node("EQ", (p, _wrap(float(f(m - 1)), lib.F32)), lib.F32)
    return if_else(last, float(f(u)), Node("FMA", (p, _wrap(float(step), lib.F32), _wrap(float(lo), lib.F32)), lib.F32))


def logspace(l, u, n=50, regular=False):
    """exp10(fma(p, step, lower)); u == pi stands for log10(pi) unless regular."""
    import numpy as np
    f = np.float32
    u = f(u)
    if not regular and u == np.uint32(0x40490fdb).view(np.float32):
        u = np.uint32(0x3efe8a6e).view(np.float32)
    lower = f(l) if n != 1 else u
    step = (u - f(l)) / f(n - 1) if n != 1 else f(0)
    return exp10(Node("FMA", (_index(n), _wrap(float(step), lib.F32), _wrap(float(lower), lib.F32)), lib.F32))


_LOGICAL_OPS = ("LT", "GT", "LE", "GE", "EQ", "NE", "IS_NAN", "IS_INF", "IS_FINITE", "IS_EQZ", "IS_NEZ", "IS_LTZ",
                "IS_GTZ")


def _compare_dtype(n):
    return n.args[0].dtype


def lower(outs, exprs, fold=None):
    """tie(outs) = tie(exprs) -> (ops, slot tensors/scalars); with fold (and
    no outs), the program that folds that expression's value."""
    slots, slot_of = [], {}

    def slot(key, value):
        if key not in slot_of:
            slot_of[key] = len(slots)
            slots.append(value)
        return slot_of[key]

    ops, memo = [], {}

    def emit(n):
        # table loads are never memoised here: a load after a store to the
        # same table must see the stored value (tie semantics); the library's
        # compiler forwards and deduplicates them
        if n.op != "LOAD" and id(n) in memo:
            return memo[id(n)]
        if n.op == "LOAD":
            s = slot(("t", n.table.data_ptr(), n.table.dtype), n.table)
            ops.append((lib.OP["LOAD"], n.dtype, s, -1, -1, 0.0))
        elif n.op == "SCALAR":
            s = slot(("s", id(n)), n)
            ops.append((lib.OP["SCALAR"], n.dtype, s, -1, -1, 0.0))
        elif n.op == "CONST":
            ops.append((lib.OP["CONST"], n.dtype, -1, -1, -1, n.imm))
        elif n.op == "INDEX":
            ops.append((lib.OP["INDEX"], n.dtype, -1, -1, -1, 0.0))
        else:
            a = [emit(x) for x in n.args] + [-1, -1, -1]
            dt = _compare_dtype(n) if n.op in _LOGICAL_OPS else n.dtype
            ops.append((lib.OP[n.op], dt, a[0], a[1], a[2], 0.0))
        memo[id(n)] = len(ops) - 1
        return memo[id(n)]

    for o, e in zip(outs, exprs):
        v = emit(e)
        dt = lib.U8 if o.dtype.is_floating_point is False else lib.F32
        s = slot(("t", o.data_ptr(), o.dtype), o)
        ops.append((lib.OP["STORE"], dt, v, s, -1, 0.0))
    if fold is not None:
        ops.append((lib.OP["FOLD"], lib.F32, emit(fold), -1, -1, 0.0))
    return ops, slots


class Program:
    def __init__(self, ops, n_slots):
        arr = (lib.Op * len(ops))(*[lib.Op(*o) for o in ops])
        h = ctypes.c_void_p()
        lib.check(lib.load().nt2g_program_create(arr, len(ops), n_slots, ctypes.byref(h)))
        self.handle = h

    def info(self):
        inf = lib.ProgramInfo()
        lib.check(lib.load().nt2g_program_info_get(self.handle, ctypes.byref(inf)))
        return inf

    def jit_source(self, precision=lib.PREC_FAST):
        """CUDA source of this program's run-time compiled kernel."""
        L, n = lib.load(), ctypes.c_size_t()
        lib.check(L.nt2g_program_jit_source(self.handle, precision, None, 0, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        lib.check(L.nt2g_program_jit_source(self.handle, precision, buf, n.value, ctypes.byref(n)))
        return buf.value.decode()

    def fold_source(self, op="sum", precision=lib.PREC_FAST):
        """CUDA source of this fold program's run-time compiled fold kernels."""
        L, n = lib.load(), ctypes.c_size_t()
        lib.check(L.nt2g_program_fold_source(self.handle, precision, lib.FOLD[op], None, 0, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        lib.check(L.nt2g_program_fold_source(self.handle, precision, lib.FOLD[op], buf, n.value, ctypes.byref(n)))
        return buf.value.decode()

    def vjp_source(self, precision=lib.PREC_FAST):
        """CUDA source of this program's reverse-mode kernel."""
        L, n = lib.load(), ctypes.c_size_t()
        lib.check(L.nt2g_program_vjp_source(self.handle, precision, None, 0, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        lib.check(L.nt2g_program_vjp_source(self.handle, precision, buf, n.value, ctypes.byref(n)))
        return buf.value.decode()

    def jit_prepare(self, precision=lib.PREC_FAST):
        """Compile and load the run-time compiled kernel now; raises Nt2gError when it is unavailable."""
        lib.check(lib.load().nt2g_program_jit_prepare(self.handle, precision))

    def __del__(self):
        try:
            if self.handle:
                lib.load().nt2g_program_destroy(self.handle)
        except Exception:
            pass


_cache = {}


def compile_program(outs, exprs, fold=None):
    ops, slots = lower(outs, exprs, fold)
    key = (tuple(ops), len(slots))
    prog = _cache.get(key)
    if prog is None:
        prog = _cache[key] = Program(ops, len(slots))
    return prog, slots


def assign(outs, exprs, precision=lib.PREC_FAST, offset=0, count=None, force_generic=False, stream=None):
    """tie(outs...) = tie(exprs...) over elements [offset, offset+count).

    force_generic: False/0 = bound fused kernel, else the run-time compiled
    kernel, else the interpreter; True/1 = compiled kernel, else interpreter;
    2 = interpreter only."""
    import torch
    outs, exprs = list(outs), list(exprs)
    prog, slots = compile_program(outs, exprs)
    args = (lib.Arg * len(slots))()
    n = None
    for i, s in enumerate(slots):
        if isinstance(s, Node):  # a SCALAR leaf
            args[i] = lib.Arg(None, s.imm, s.dtype, 1)
        else:
            n = s.numel() if n is None else min(n, s.numel())
            args[i] = lib.Arg(s.data_ptr(), 0.0, lib.U8 if s.dtype == torch.uint8 else lib.F32, 0)
    if count is None:
        count = n - offset
        _check_generative_sizes(exprs, count)
    lib.check(lib.load().nt2g_eval(prog.handle, args, len(slots), offset, count, precision,
                                   int(force_generic), lib._stream(stream)))
    return prog


def _args_of(slots):
    import torch
    args = (lib.Arg * len(slots))()
    n = None
    for i, s in enumerate(slots):
        if isinstance(s, Node):  # a SCALAR leaf
            args[i] = lib.Arg(None, s.imm, s.dtype, 1)
        else:
            n = s.numel() if n is None else min(n, s.numel())
            args[i] = lib.Arg(s.data_ptr(), 0.0, lib.U8 if s.dtype == torch.uint8 else lib.F32, 0)
    return args, n


def _slot_of(slots, x):
    import torch
    for i, s in enumerate(slots):
        if isinstance(x, torch.Tensor):
            if not isinstance(s, Node) and s.data_ptr() == x.data_ptr() and s.dtype == x.dtype:
                return i
        elif s is x:
            return i
    raise ValueError("not an argument of the program")


def vjp(outs, exprs, cotangents, inputs, precision=lib.PREC_FAST, stream=None):
    """Reverse mode of tie(outs...) = tie(exprs...) (nt2g_program_vjp):
    cotangents holds one float table per output (None: zero); returns the
    gradient with respect to each of `inputs` -- a float table (a fresh
    table of its shape) or a Scalar leaf (a 0-d float64 tensor: the gradient
    summed over the elements); zeros for an input the program does not read.  Forward values are recomputed on the fly;
    the output tables are not written."""
    import torch
    outs, exprs = list(outs), list(exprs)
    prog, slots = compile_program(outs, exprs)
    args, n = _args_of(slots)
    ns = len(slots)
    ct, tg = (ctypes.c_void_p * ns)(), (ctypes.c_void_p * ns)()
    for o, c in zip(outs, cotangents):
        if c is not None:
            ct[_slot_of(slots, o)] = c.data_ptr()
    dev = next(s.device for s in slots if not isinstance(s, Node))
    res, scalars = [], []
    for x in inputs:
        try:
            k = _slot_of(slots, x)
        except ValueError:  # the program does not read it: a zero gradient
            res.append(torch.zeros_like(x) if isinstance(x, torch.Tensor)
                       else torch.zeros((), dtype=torch.float64, device=dev))
            continue
        if isinstance(x, torch.Tensor):
            g = torch.empty_like(x)
            tg[k] = g.data_ptr()
            res.append(g)
        else:
            scalars.append((len(res), k))
            res.append(None)
    sg = torch.zeros(max(ns, 1), dtype=torch.float64, device=dev) if scalars else None
    nb = ctypes.c_size_t()
    L = lib.load()
    lib.check(L.nt2g_program_vjp_workspace_size(prog.handle, n, ctypes.byref(nb)))
    ws = torch.empty(max(nb.value, 16), dtype=torch.uint8, device=dev)
    lib.check(L.nt2g_program_vjp(prog.handle, args, ns, n, ct, tg, lib._ptr(sg), precision, lib._ptr(ws), ws.numel(),
                                 lib._stream(stream)))
    for i, k in scalars:
        res[i] = sg[k]
    return res


def batch_item(outs, exprs):
    """A program item of a batch (nt2g_batch_item, NT2G_BATCH_PROGRAM):
    tie(outs...) = tie(exprs...) over the whole tables.  Returns (item,
    program, args): args must stay alive until nt2g_batch_create returns, the
    program (also held by this module's cache) as long as the batch."""
    outs, exprs = list(outs), list(exprs)
    prog, slots = compile_program(outs, exprs)
    args, n = _args_of(slots)
    if n is None:
        n = _generative_sizes(exprs[0]).pop()
    _check_generative_sizes(exprs, n)
    it = lib.BatchItem()
    it.expr, it.n, it.n_args = lib.BATCH_PROGRAM, n, len(slots)
    it.program = prog.handle.value
    it.args = ctypes.cast(args, ctypes.POINTER(lib.Arg))
    return it, prog, args


def wmean(a, w, shape=None, precision=lib.PREC_FAST):
    """NT2's wmean(a, w, dim) (reduction/functions/expr/wmean.hpp):
    rec(globalsum(w)) times the fold of a .* w along the view's inner
    dimension (shape = (lo, inner, hi), default every element), the product
    folded in one pass and the scaling by this library's multiply."""
    import numpy as np
    import torch
    f = np.float32(1.0) / np.float32(fold(Table(w), "sum", precision=precision).item())
    s = fold(Table(a) * Table(w), "sum", shape, precision=precision)
    out = torch.empty_like(s)
    assign([out], [Scalar(float(f)) * Table(s)], precision=precision)
    return out


def asump(a, p, shape=None, precision=lib.PREC_FAST):
    """NT2's asump(a, p, dim) = sum(pow_abs(a, p), dim) of a device table viewed as
    shape = (lo, inner, hi) (default every element): pow(abs(a), p) folded in one pass."""
    return fold(pow(abs_(Table(a)), float(p)), "sum", shape, precision=precision)


def normp(a, p, shape=None, precision=lib.PREC_FAST):
    """NT2's normp(a, p, dim) = pow(asump(a, p, dim), rec(p)), rec(p) in float."""
    import numpy as np
    import torch
    s = asump(a, p, shape, precision)
    out = torch.empty_like(s)
    assign([out], [pow(Table(s), float(np.float32(1.0) / np.float32(p)))], precision=precision)
    return out


def nanasum2(a, shape=None, precision=lib.PREC_FAST):
    """NT2's nanasum2(a, dim) = sum(if_zero_else(is_nan(a), sqr_abs(a)), dim), in one pass."""
    t = Table(a)
    return fold(if_else(is_nan(t), 0.0, t * t), "sum", shape, precision=precision)


def median(a, shape=None):
    """NT2's median(a, dim) of a device table viewed as shape = (lo, inner, hi)
    along inner (default every element: globalmedian); the same under either
    arithmetic policy (an order statistic, or meanof of two)."""
    return lib.median(a, *(shape or (1, a.numel(), 1)), "median")


def medianad(a, shape=None):
    """NT2's medianad(a, dim) = median(abs(a - median(a, dim)), dim)."""
    return lib.median(a, *(shape or (1, a.numel(), 1)), "medianad")


def batch_source(programs, precision=lib.PREC_FAST, block_threads=256):
    """CUDA source of the batch kernel that links these programs."""
    L, n = lib.load(), ctypes.c_size_t()
    hs = (ctypes.c_void_p * len(programs))(*[p.handle.value for p in programs])
    lib.check(L.nt2g_batch_source(hs, len(programs), precision, block_threads, None, 0, ctypes.byref(n)))
    buf = ctypes.create_string_buffer(n.value)
    lib.check(L.nt2g_batch_source(hs, len(programs), precision, block_threads, buf, n.value, ctypes.byref(n)))
    return buf.value.decode()


def fold(e, op="sum", shape=None, precision=lib.PREC_FAST, index=False, out64=False, stream=None):
    """NT2's fold of an expression along one dimension in one pass
    (nt2g_eval_fold): e's value at every element is computed inside the fold
    kernels, no temporary table.  shape = (lo, inner, hi), the column-major
    view folded over inner (default: every element, lo = hi = 1).  Returns the
    float results (lo*hi), then the 0-based first index of max/min (index=True)
    and the FP64 results (out64=True) when asked."""
    import torch
    prog, slots = compile_program([], [], fold=e)
    args, n = _args_of(slots)
    if shape is None:
        if n is None:
            n = _generative_sizes(e).pop()
        shape = (1, n, 1)
    lo, inner, hi = (int(v) for v in shape)
    dev = next((s.device for s in slots if not isinstance(s, Node)), torch.device("cuda"))
    nb = ctypes.c_size_t()
    lib.check(lib.load().nt2g_fold_workspace_size(lo, inner, hi, ctypes.byref(nb)))
    ws = torch.empty(max(nb.value, 16), dtype=torch.uint8, device=dev)
    out = torch.empty(lo * hi, dtype=torch.float32, device=dev)
    idx = torch.empty(lo * hi, dtype=torch.int64, device=dev) if index else None
    o64 = torch.empty(lo * hi, dtype=torch.float64, device=dev) if out64 else None
    lib.check(lib.load().nt2g_eval_fold(prog.handle, args, len(slots), lo, inner, hi, lib.FOLD[op], precision,
                                        lib._ptr(ws), ws.numel(), lib._ptr(out), lib._ptr(idx), lib._ptr(o64),
                                        lib._stream(stream)))
    res = [out] + ([idx] if index else []) + ([o64] if out64 else [])
    return res[0] if len(res) == 1 else tuple(res)
