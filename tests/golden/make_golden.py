"""Regenerate nt2_unit_vectors.json from NT2's own unit tests.

Reads the cited NT2_TEST_ULP_EQUAL / NT2_TEST_EQUAL lines of the reference's
test sources as text (nothing of the reference is compiled or run), evaluates
the NT2 constant spellings they use (Inf, Mzero, Half, Exp_1, T(0.4795...),
...) for T = float, and writes one record per known answer:
{fn, x, expected, tol_nt2ulp, source}.  The float tolerance is in NT2's ulp
unit (half a standard ulp).

Usage (needs the reference checkout):  python tests/golden/make_golden.py /path/to/nt2
"""
import json
import math
import os
import re
import sys

import numpy as np

# (file, first line, last line) inside the NT2 tree; each holds ULP checks of
# one scalar float functor
SOURCES = [
    ("modules/core/exponential/unit/scalar/exp.cpp", 40, 46),
    ("modules/core/exponential/unit/simd/log.cpp", 44, 51),
    ("modules/core/euler/unit/scalar/erfc.cpp", 42, 53),
    ("modules/core/statistics/unit/scalar/normcdf.cpp", 31, 36),
    ("modules/core/statistics/unit/scalar/fastnormcdf.cpp", 26, 31),
    ("modules/core/exponential/unit/scalar/exp2.cpp", 42, 48),
    ("modules/core/exponential/unit/scalar/exp10.cpp", 40, 46),
    ("modules/core/exponential/unit/scalar/expm1.cpp", 40, 46),
    ("modules/core/exponential/unit/scalar/log2.cpp", 39, 48),
    ("modules/core/exponential/unit/scalar/log10.cpp", 39, 45),
    ("modules/core/trigonometric/unit/scalar/sin.cpp", 44, 52),
    ("modules/core/trigonometric/unit/scalar/cos.cpp", 45, 55),
    ("modules/core/trigonometric/unit/scalar/tan.cpp", 41, 49),
    ("modules/core/trigonometric/unit/scalar/sinpi.cpp", 45, 54),
    ("modules/core/trigonometric/unit/scalar/cospi.cpp", 45, 54),
    ("modules/core/hyperbolic/unit/scalar/sinh.cpp", 40, 44),
    ("modules/core/hyperbolic/unit/scalar/cosh.cpp", 37, 41),
    ("modules/core/hyperbolic/unit/scalar/tanh.cpp", 38, 44),
    ("modules/core/trigonometric/unit/scalar/asin.cpp", 45, 53),
    ("modules/core/trigonometric/unit/scalar/acos.cpp", 46, 54),
    ("modules/core/trigonometric/unit/scalar/atan.cpp", 45, 53),
    ("modules/core/hyperbolic/unit/scalar/asinh.cpp", 42, 46),
    ("modules/core/hyperbolic/unit/scalar/asinh.cpp", 49, 49),
    ("modules/core/hyperbolic/unit/scalar/acosh.cpp", 37, 42),
    ("modules/core/hyperbolic/unit/scalar/atanh.cpp", 38, 44),
    ("modules/core/exponential/unit/scalar/cbrt.cpp", 40, 47),
    ("modules/core/trigonometric/unit/scalar/cot.cpp", 42, 51),
    ("modules/core/trigonometric/unit/scalar/sec.cpp", 42, 50),
    ("modules/core/trigonometric/unit/scalar/csc.cpp", 42, 51),
    ("modules/core/trigonometric/unit/scalar/sind.cpp", 41, 51),
    ("modules/core/trigonometric/unit/scalar/cosd.cpp", 42, 52),
    ("modules/core/trigonometric/unit/scalar/tand.cpp", 40, 50),
    # whole files from here on (1-200: every float ULP_EQUAL line they hold)
    ("modules/core/trigonometric/unit/scalar/tanpi.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/proper_tanpi.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/cotpi.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/cotd.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/secpi.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/cscpi.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/secd.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/cscd.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/sinc.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/sincpi.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/acotd.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/asec.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/acsc.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/asind.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/acosd.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/atand.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/asecd.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/acscd.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/asinpi.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/acospi.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/atanpi.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/acot.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/indeg.cpp", 1, 200),
    ("modules/core/trigonometric/unit/scalar/inrad.cpp", 1, 200),
    ("modules/core/hyperbolic/unit/scalar/coth.cpp", 1, 200),
    ("modules/core/hyperbolic/unit/scalar/sinhc.cpp", 1, 200),
    ("modules/core/hyperbolic/unit/scalar/sech.cpp", 1, 200),
    ("modules/core/hyperbolic/unit/scalar/csch.cpp", 1, 200),
    ("modules/core/hyperbolic/unit/scalar/asech.cpp", 1, 200),
    ("modules/core/hyperbolic/unit/scalar/acsch.cpp", 1, 200),
    ("modules/core/hyperbolic/unit/scalar/acoth.cpp", 1, 200),
    ("modules/core/euler/unit/scalar/erf.cpp", 1, 200),
    ("modules/core/euler/unit/scalar/erfcx.cpp", 1, 200),
    ("modules/core/euler/unit/scalar/gamma.cpp", 1, 200),
    ("modules/core/euler/unit/scalar/gammaln.cpp", 1, 200),
    ("modules/core/euler/unit/scalar/digamma.cpp", 1, 200),
    ("modules/core/euler/unit/scalar/signgam.cpp", 1, 200),
    ("modules/core/euler/unit/scalar/dawson.cpp", 1, 200),
    ("modules/core/euler/unit/scalar/spence.cpp", 1, 200),
    ("modules/core/euler/unit/scalar/stirling.cpp", 1, 200),
    ("modules/core/euler/unit/scalar/erfinv.cpp", 1, 200),
    ("modules/core/euler/unit/scalar/erfcinv.cpp", 1, 200),
    ("modules/core/exponential/unit/scalar/expx2.cpp", 1, 200),
    ("modules/core/exponential/unit/scalar/exprecneg.cpp", 1, 200),
    ("modules/core/exponential/unit/scalar/exprecnegc.cpp", 1, 200),
    ("modules/core/exponential/unit/scalar/sqrt1pm1.cpp", 1, 200),
    ("modules/core/exponential/unit/scalar/realsqrt.cpp", 1, 200),
    ("modules/core/exponential/unit/scalar/reallog.cpp", 1, 200),
]

E = float(np.float32(math.e))
CONST = {
    "Inf": math.inf, "Minf": -math.inf, "Nan": math.nan, "Zero": 0.0, "Mzero": -0.0, "One": 1.0, "Mone": -1.0,
    "Half": 0.5, "Two": 2.0, "Ten": 10.0, "Exp_1": E, "Eps": float(np.finfo(np.float32).eps),
    "Mhalf": -0.5, "Quarter": 0.25,
    # NT2's float pi constants by bit pattern (boost/simd/constant/constants/*.hpp)
    "Pi": float(np.uint32(0x40490fdb).view(np.float32)), "Pio_2": float(np.uint32(0x3fc90fdb).view(np.float32)),
    "Pio_4": float(np.uint32(0x3f490fdb).view(np.float32)),
    "Sqrt_2o_2": float(np.uint32(0x3f3504f3).view(np.float32)),
    "Pio_6": float(np.uint32(0x3f060a92).view(np.float32)), "Pio_3": float(np.uint32(0x3f860a92).view(np.float32)),
    "Twopio_3": float(np.uint32(0x40060a92).view(np.float32)),
    "Threepio_4": float(np.uint32(0x4016cbe4).view(np.float32)),
    "Sqrt_2": float(np.uint32(0x3fb504f3).view(np.float32)), "Valmax": float(np.finfo(np.float32).max),
    "_45": 45.0, "_90": 90.0, "_135": 135.0, "_180": 180.0,
    "Mindenormal": float(np.uint32(1).view(np.float32)), "Mtwo": -2.0, "Maxflint": 16777216.0, "Valmin": -float(np.finfo(np.float32).max),
    "Three": 3.0, "Four": 4.0, "Five": 5.0, "Mthree": -3.0,
    "Log_2": float(np.uint32(0x3f317218).view(np.float32)),
    "Invexp_1": float(np.uint32(0x3ebc5ab2).view(np.float32)),
    "Pi2o_6": float(np.uint32(0x3fd28d33).view(np.float32)),
    "Invsqrt_2pi": float(np.uint32(0x3ecc422a).view(np.float32)),
}


def _value(expr):
    expr = re.sub(r"\s+<", "<", expr.strip())
    if expr.startswith("-nt2::"):  # a negated constant
        return -_value(expr[1:])
    m = re.fullmatch(r"(?:nt2|boost::simd)::(\w+)<\w+>\(\)", expr)
    if m:
        return CONST[m.group(1)]
    m = re.fullmatch(r"[-+]?[0-9.]+[eE][-+]?[0-9]+", expr)
    if m:  # a bare double literal, converted to the float r_t
        return float(np.float32(float(expr)))
    m = re.fullmatch(r"T\(\s*1\s*-\s*([0-9.]+)\s*\)", expr)
    if m:  # a double difference converted to T
        return float(np.float32(1.0 - float(m.group(1))))
    m = re.fullmatch(r"T\(\s*([-+0-9.eE]+)\s*\)", expr)
    if m:
        return float(np.float32(float(m.group(1))))
    m = re.fullmatch(r"nt2::One<\w+>\(\)\s*/\s*nt2::Exp_1<\w+>\(\)", expr)
    if m:
        return float(np.float32(1.0) / np.float32(E))
    m = re.fullmatch(r"nt2::One<\w+>\(\)\s*/\s*nt2::Exp_1<\w+>\(\)\s*-\s*nt2::One<\w+>\(\)", expr)
    if m:  # float arithmetic as the test writes it
        return float(np.float32(np.float32(1.0) / np.float32(E)) - np.float32(1.0))
    m = re.fullmatch(r"nt2::Exp_1<\w+>\(\)\s*-\s*nt2::One<\w+>\(\)", expr)
    if m:
        return float(np.float32(E) - np.float32(1.0))
    m = re.fullmatch(r"nt2::One<\w+>\(\)\s*/\s*10", expr)
    if m:
        return float(np.float32(1.0) / np.float32(10.0))
    m = re.fullmatch(r"iT\(\s*(-?[0-9]+)\s*\)", expr)
    if m:  # an integer argument (nthroot's n)
        return float(int(m.group(1)))
    m = re.fullmatch(r"[-+]?[0-9]+(\.[0-9]*)?", expr)
    if m:  # an integer or decimal literal converted to the float r_t
        return float(np.float32(float(expr)))
    m = re.fullmatch(r"(-?)T\(([0-9]+)\)\s*/\s*(?:T\()?([0-9]+)\)?", expr)
    if m:  # a quotient in float: T(1)/T(4), -T(1)/6
        q = np.float32(float(m.group(2))) / np.float32(float(m.group(3)))
        return float(-q if m.group(1) else q)
    m = re.fullmatch(r"T\(2\)\s*/\s*\(nt2::Pi<\w+>\(\)\)", expr)
    if m:
        return float(np.float32(2.0) / np.float32(CONST["Pi"]))
    m = re.fullmatch(r"nt2::rec\(nt2::(Eps|Exp_1)<\w+>\(\)\)", expr)
    if m:
        return float(np.float32(1.0) / np.float32(CONST[m.group(1)]))
    m = re.fullmatch(r"((?:nt2|boost::simd)::\w+<\w+>\(\))\s*([-+])\s*((?:nt2|boost::simd)::\w+<\w+>\(\))", expr)
    if m:  # a sum or difference of two constants, in float
        a, b = np.float32(_value(m.group(1))), np.float32(_value(m.group(3)))
        return float(a + b if m.group(2) == "+" else a - b)
    raise ValueError(f"unhandled NT2 constant spelling: {expr!r}")


PAT = re.compile(r"NT2_TEST_ULP_EQUAL\(\s*(\w+)\((.*?)\)\s*,\s*(.*?)\s*,\s*([0-9.]+)\s*\);")
# two-argument functors: pow(a, b)
ARG = r"((?:[^,()]|\([^()]*\))*)"
PAT2 = re.compile(r"NT2_TEST_ULP_EQUAL\(\s*(pow|atan2d?|hypot|logspace_add|logspace_sub|beta|betaln|nthroot|expni|gammainc|gammaincinv|normpdf|norminv|expcdf|exppdf|expinv|logncdf|lognpdf|logninv|caucdf|cauinv|caupdf|evcdf|evpdf|evinv)\(" + ARG + r",\s*" + ARG +
                  r"\)\s*,\s*(.*?)\s*,\s*([0-9.]+)\s*\);")
# NT2's distribution functions (statistics/unit/scalar): their one-argument
# known answers above, the two-argument ones (fn(x, p1)) in the second pass
STAT_FNS = ("normpdf", "norminv", "expcdf", "exppdf", "expinv", "logncdf", "lognpdf", "logninv", "unifcdf", "unifpdf",
            "unifinv", "caucdf", "cauinv", "caupdf", "evcdf", "evpdf", "evinv")
SOURCES += [(f"modules/core/statistics/unit/scalar/{f}.cpp", 1, 200) for f in STAT_FNS]
SOURCES2 = [("modules/core/exponential/unit/scalar/pow.cpp", 43, 53),
            ("modules/core/trigonometric/unit/scalar/atan2.cpp", 47, 61),
            ("modules/boost/simd/base/unit/arithmetic/scalar/hypot.cpp", 42, 52),
            ("modules/core/trigonometric/unit/scalar/atan2d.cpp", 46, 60),
            ("modules/core/exponential/unit/scalar/logspace_add.cpp", 1, 200),
            ("modules/core/exponential/unit/scalar/logspace_sub.cpp", 1, 200),
            ("modules/core/euler/unit/scalar/beta.cpp", 1, 200),
            ("modules/core/euler/unit/scalar/betaln.cpp", 1, 200),
            ("modules/core/exponential/unit/scalar/nthroot.cpp", 1, 200),
            ("modules/core/euler/unit/scalar/expni.cpp", 1, 200),
            ("modules/core/euler/unit/scalar/gammainc.cpp", 1, 200),
            ("modules/core/euler/unit/scalar/gammaincinv.cpp", 1, 200)] + \
           [(f"modules/core/statistics/unit/scalar/{f}.cpp", 1, 200) for f in STAT_FNS]
# expected values that are themselves results of NT2 functors (sin(Pio_4)/Pio_4)
# are left out: they would pin the oracle to itself; so are values from
# Boost.Math (boost::math::digamma), which is not part of the reference
SELF_REFERENCE = re.compile(r"nt2::(sin|sinpi|cos|exp)\(|boost::math::")


# exact functors: NT2_TEST_EQUAL(fn(args), expected) in the float (_real) test
# case of boost.simd's unit tests (the integer cases are out of scope)
EQ = re.compile(r"NT2_TEST_EQUAL\(\s*(\w+)\(" + r"((?:[^,()]|\([^()]*\))*)" + r"(?:,\s*((?:[^,()]|\([^()]*\))*))?\)\s*,\s*(.*?)\s*\);")
EQ_SOURCES = [f"modules/boost/simd/base/unit/arithmetic/scalar/{f}.cpp" for f in
              ("floor", "ceil", "trunc", "round", "round2even", "oneplus", "oneminus", "minusone", "dist", "average",
               "sqr_abs", "mod", "rem", "minmod", "divfloor", "divceil", "divfix", "divround",
               "divround2even")] + [f"modules/boost/simd/base/unit/ieee/scalar/{f}.cpp" for f in ("frac", "sign", "signnz",
                                                                                           "copysign", "maxnum", "minnum",
                                                                                           "maxmag", "minmag", "negate")] + \
             ["modules/core/exponential/unit/scalar/pow2.cpp"]


def _real_block_equalities(root, rel):
    out, skipped, inside = [], 0, False
    for ln, line in enumerate(open(os.path.join(root, rel)).read().splitlines(), 1):
        if "NT2_TEST_CASE_TPL" in line:
            inside = "_real" in line or "REAL_TYPES" in line
            continue
        m = EQ.search(line) if inside else None
        if not m:
            continue
        fn, a0, a1, exp = m.groups()
        if (a1 is not None) != (fn in ("copysign", "dist", "average", "mod", "rem", "pow2", "maxnum", "minnum",
                                                 "maxmag", "minmag", "minmod", "negate", "divfloor",
                                                 "divceil", "divfix", "divround", "divround2even")):
            continue  # another arity (round(x, n) rounds to n digits): not these functors
        try:
            rec = dict(fn=fn, x=_value(a0), expected=_value(exp), tol_nt2ulp=0.0, source=f"{rel}:{ln}")
            if a1 is not None:
                rec["y"] = _value(a1)
        except (ValueError, KeyError):
            skipped += 1
            continue
        out.append(rec)
    return out, skipped


def main(root):
    out = []
    for rel, lo, hi in SOURCES:
        lines = open(os.path.join(root, rel)).read().splitlines()
        for ln in range(lo, min(hi, len(lines)) + 1):
            if lines[ln - 1].lstrip().startswith("//"):
                continue  # a check the test leaves commented out
            m = PAT.search(lines[ln - 1])
            if not m:
                continue
            fn, arg, exp, tol = m.groups()
            if SELF_REFERENCE.search(exp):
                continue
            if fn in STAT_FNS and "," in arg:
                continue  # a two-argument form: the second pass below
            try:
                out.append(dict(fn=fn, x=_value(arg), expected=_value(exp), tol_nt2ulp=float(tol),
                                source=f"{rel}:{ln}"))
            except (ValueError, KeyError):
                if fn not in STAT_FNS:
                    raise
                continue  # a table variable (expcdf(a), r): not a scalar known answer
    for rel, lo, hi in SOURCES2:
        lines = open(os.path.join(root, rel)).read().splitlines()
        for ln in range(lo, min(hi, len(lines)) + 1):
            m = PAT2.search(lines[ln - 1])
            if not m:
                continue
            fn, a0, a1, exp, tol = m.groups()
            try:
                out.append(dict(fn=fn, x=_value(a0), y=_value(a1), expected=_value(exp), tol_nt2ulp=float(tol),
                                source=f"{rel}:{ln}"))
            except (ValueError, KeyError):
                continue  # a loop variable (betaln(T(i), T(6-i))): the table below
    # betaln(i, 6 - i) for i = 1..5 against the table r[5], 0.5 NT2-ulp
    rel = "modules/core/euler/unit/scalar/betaln.cpp"
    lines = open(os.path.join(root, rel)).read().splitlines()
    body = lines[37][lines[37].index("{") + 1:lines[37].index("}")]
    vals = [float(np.float32(float(v.strip()[2:-1]))) for v in body.split(",")]
    assert len(vals) == 5, vals
    for i in range(1, 6):
        out.append(dict(fn="betaln", x=float(i), y=float(6 - i), expected=vals[i - 1], tol_nt2ulp=0.5,
                        source=f"{rel}:38-42"))
    skipped = 0
    for rel in EQ_SOURCES:
        recs, k = _real_block_equalities(root, rel)
        out += recs
        skipped += k
    print(f"exact functors: {skipped} lines with expressions this parser does not evaluate were left out")
    # normcdf on _(-5, 1, 5) against the 11-value table r0, 5 NT2-ulp
    rel = "modules/core/statistics/unit/scalar/normcdf.cpp"
    lines = open(os.path.join(root, rel)).read().splitlines()
    text = " ".join(lines[53:57])  # lines 54-57: r0 = nt2::cons<T>( ... );
    body = text[text.index("cons<T>(") + len("cons<T>("):text.index(");")]
    vals = [float(np.float32(float(v))) for v in body.replace(")", "").split(",") if v.strip()]
    assert len(vals) == 11, vals
    for k, v in enumerate(vals):
        out.append(dict(fn="normcdf", x=float(k - 5), expected=v, tol_nt2ulp=5.0, source=f"{rel}:53-61"))
    # sum / dot / globalsum known answers (exact integers)
    out.append(dict(fn="sum_ones", n=133, expected=133.0, source="modules/arch/openmp/unit/functions/sum.cpp:40-45"))
    out.append(dict(fn="globalsum_1_to_9", expected=45.0,
                    source="modules/core/reduction/unit/table/globalsum.cpp:24-25"))
    out.append(dict(fn="globalsum_1_to_8", expected=36.0,
                    source="modules/core/reduction/unit/table/globalsum.cpp:27-28"))
    out.append(dict(fn="dot_5x3_i_minus_j", expected=float(sum((i - j) ** 2 for i in range(1, 6) for j in range(1, 4))),
                    source="modules/core/reduction/unit/table/dot.cpp:46-59,73"))
    # median / medianad of the 4 x 3 table y(i, j) = 4(j - 1) + i along each
    # dimension (NT2_TEST_EQUAL, exact), and of [ones(4,1) zeros(4,1) ones(4,1)]
    # along 2; the tables are column-major, [lo, inner, hi] as the fold ABI
    y = [float(k) for k in range(1, 13)]
    rel = "modules/core/reduction/unit/table/median.cpp"
    for dim, shape, exp, lines in ((1, (1, 4, 3), [2.5, 6.5, 10.5], "42,48-53"), (2, (4, 3, 1), [5., 6., 7., 8.], "43,54-56"),
                                   (3, (12, 1, 1), y, "57-59"), (4, (12, 1, 1), y, "60-62")):
        out.append(dict(fn="median", x=y, shape=list(shape), expected=exp, source=f"{rel}:{lines}"))
    out.append(dict(fn="median", x=[1.] * 4 + [0.] * 4 + [1.] * 4, shape=[4, 3, 1], expected=[1.] * 4,
                    source=f"{rel}:64-77"))
    rel = "modules/core/reduction/unit/table/medianad.cpp"
    for dim, shape, exp, lines in ((1, (1, 4, 3), [1.] * 3, "41,48-51"), (2, (4, 3, 1), [4.] * 4, "42,53-54"),
                                   (3, (12, 1, 1), [0.] * 12, "55-56"), (4, (12, 1, 1), [0.] * 12, "58-59")):
        out.append(dict(fn="medianad", x=y, shape=list(shape), expected=exp, source=f"{rel}:{lines}"))
    # trapz of reshape(1:15, 5, 3): over every element, along dimension 1 and
    # along dimension 2 (unit spacing, the x1 = 1:3 form), exact
    rel = "modules/core/reduction/unit/table/trapz.cpp"
    y15 = [float(k) for k in range(1, 16)]
    for shape, exp, lines in (((1, 15, 1), [112.0], "34-38"), ((1, 5, 3), [12.0, 32.0, 52.0], "31,40-42"),
                              ((5, 3, 1), [12.0, 14.0, 16.0, 18.0, 20.0], "29,32,48-50")):
        out.append(dict(fn="trapz", x=y15, shape=list(shape), expected=exp, source=f"{rel}:{lines}"))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "nt2_unit_vectors.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1, default=lambda v: v)
    print(f"wrote {len(out)} records to {path}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
