"""Run-time compiled kernels of generic programs.

A program that binds none of the fused kernels is compiled by NVRTC into a
straight-line kernel (NT2's planned per-expression CUDA generator,
tools/external_kernel/backend.cpp:32-52 and tools/kernel_gen/kernel_gen.cpp:8-113).
Each of its statements is the interpreter's arithmetic for the same
instruction, so the two kernels must agree bit for bit; under the NT2 policy
both must equal the oracle's restatement of NT2's CPU evaluation.
"""
import numpy as np
import pytest
import torch

from nt2_gb300 import expr as E
from helpers import bs_inputs

pytestmark = pytest.mark.gpu

JIT, INTERP = 1, 2
SIGMA, R = 0.30, 0.02


def _bits_equal(a, b):
    """Bitwise equality, with any NaN equal to any NaN."""
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype == np.float32:
        nan = np.isnan(a) & np.isnan(b)
        return bool(np.all((a.view(np.uint32) == b.view(np.uint32)) | nan))
    return bool(np.array_equal(a, b))


_UNARY_F = ["NEG", "ABS", "SQR", "SQRT", "REC", "EXP", "LOG", "LOG1P", "ERFC", "NORMCDF", "FASTNORMCDF", "EXP2",
            "EXP10", "EXPM1", "LOG2", "LOG10", "SIN", "COS", "TAN", "SINPI", "COSPI",
            "SINH", "COSH", "TANH", "ASIN", "ACOS", "ATAN", "ASINH", "ACOSH", "ATANH", "CBRT",
            "COT", "SEC", "CSC", "SIND", "COSD", "TAND", "TANPI", "COTPI", "COTD", "SECPI", "CSCPI", "SECD", "CSCD",
            "SINC", "SINCPI", "ACOTD", "ASEC", "COTH", "SINHC", "ACSC", "ASECH", "ACOTH", "ACSCH",
            "ERF", "ERFCX", "EXPX2", "GAMMA", "GAMMALN", "EXPRECNEG", "EXPRECNEGC", "SQRT1PM1",
            "ERFINV", "ERFCINV", "FLOOR", "CEIL", "TRUNC", "ROUND", "ROUND2EVEN", "FRAC", "SIGN", "SIGNNZ"]
_BINARY_F = ["ADD", "SUB", "MUL", "DIV", "MIN", "MAX", "POW", "ATAN2", "HYPOT", "COPYSIGN"]
_CMP = ["LT", "GT", "LE", "GE", "EQ", "NE"]


def _random_float_program(rng, leaves, depth_ops=24):
    """A random DAG over the float leaves using every float opcode family."""
    vals = list(leaves)

    def pick():
        return vals[int(rng.integers(len(vals)))]

    def cond():
        op = _CMP[int(rng.integers(len(_CMP)))]
        a, b = pick(), pick() if rng.random() < 0.7 else float(np.float32(rng.uniform(-2, 2)))
        return E._bin(op, a, b)

    for _ in range(depth_ops):
        k = rng.random()
        if k < 0.35:
            op = _UNARY_F[int(rng.integers(len(_UNARY_F)))]
            v = E.Node(op, (pick(),), 0)
        elif k < 0.7:
            op = _BINARY_F[int(rng.integers(len(_BINARY_F)))]
            b = pick() if rng.random() < 0.8 else float(np.float32(rng.uniform(-3, 3)))
            v = E._bin(op, pick(), b)
        elif k < 0.8:
            v = (E.fma if rng.random() < 0.5 else E.fnms)(pick(), pick(), pick())
        elif k < 0.88:
            v = E.if_else(cond(), pick(), pick())
        elif k < 0.94:
            v = (E.selinc if rng.random() < 0.5 else E.seldec)(cond(), pick())
        else:
            v = E.if_zero_else_one(cond(), 0)
        vals.append(v)
    return vals[-1], vals[-2], cond()


def _float_tables(dev, n, k, rng):
    return [torch.from_numpy(rng.uniform(-4, 4, n).astype(np.float32)).to(dev) for _ in range(k)]


@pytest.mark.parametrize("prec", [0, 1], ids=["fast", "nt2"])
@pytest.mark.parametrize("seed", range(6))
def test_random_float_programs_match_interpreter(lib, dev, prec, seed):
    rng = np.random.default_rng(100 + seed)
    n = 4099
    ins = _float_tables(dev, n + 1, 3, rng)
    leaves = [E.Table(t) for t in ins] + [E.Scalar(float(np.float32(rng.uniform(-2, 2))))]
    e1, e2, c = _random_float_program(rng, leaves)
    for offset in (0, 1):  # offset 1 breaks 16-byte alignment: the element-wise path
        outs = {m: [torch.full((n + 1,), 7.0, device=dev) for _ in range(3)] for m in (JIT, INTERP)}
        for m in (JIT, INTERP):
            prog = E.assign(outs[m], [e1, e2, c], precision=prec, offset=offset, count=n - offset,
                            force_generic=m)
        assert prog.info().kernel_name == b"generic"
        prog.jit_prepare(prec)  # raises if the compiled kernel is unavailable
        torch.cuda.synchronize()
        for a, b in zip(outs[JIT], outs[INTERP]):
            assert _bits_equal(a.cpu().numpy(), b.cpu().numpy()), (seed, offset)
        untouched = outs[JIT][0].cpu().numpy()[[0, n] if offset else [n]]
        assert (untouched == 7.0).all()  # nothing outside the range


_BINARY_U = ["ADD", "SUB", "MUL", "MIN", "MAX", "ADDS"]


@pytest.mark.parametrize("seed", range(4))
def test_random_uint8_programs_match_interpreter(lib, dev, seed):
    rng = np.random.default_rng(200 + seed)
    n = 10003
    ins = [torch.from_numpy(rng.integers(0, 256, n, dtype=np.uint8)).to(dev) for _ in range(3)]
    vals = [E.Table(t) for t in ins] + [E.Scalar(int(rng.integers(0, 256)), 1)]
    for _ in range(20):
        k = rng.random()
        pick = lambda: vals[int(rng.integers(len(vals)))]  # noqa: E731
        if k < 0.5:
            op = _BINARY_U[int(rng.integers(len(_BINARY_U)))]
            b = pick() if rng.random() < 0.8 else int(rng.integers(0, 256))
            v = E._bin(op, pick(), b)
        elif k < 0.6:
            v = E.Node(["NEG", "ABS", "SQR"][int(rng.integers(3))], (pick(),), 1)
        elif k < 0.75:
            v = E.if_else(E._bin(_CMP[int(rng.integers(6))], pick(), pick()), pick(), pick())
        elif k < 0.9:
            v = (E.selinc if rng.random() < 0.5 else E.seldec)(E._bin(_CMP[int(rng.integers(6))], pick(), pick()),
                                                             pick())
        else:
            v = E.if_zero_else_one(E._bin(_CMP[int(rng.integers(6))], pick(), pick()), 1)
        vals.append(v)
    outs = {m: [torch.zeros(n, dtype=torch.uint8, device=dev) for _ in range(2)] for m in (JIT, INTERP)}
    for m in (JIT, INTERP):
        prog = E.assign(outs[m], [vals[-1], vals[-3]], force_generic=m)
    prog.jit_prepare(0)
    torch.cuda.synchronize()
    for a, b in zip(outs[JIT], outs[INTERP]):
        assert _bits_equal(a.cpu().numpy(), b.cpu().numpy()), seed


def _bs_generic(S, K, T, sig, r):
    sq = E.sqrt(T)
    d1 = (E.log(S / K) + E.fma(E.sqr(sig), 0.5, r) * T) / (sig * sq)
    d2 = E.fnms(sig, sq, d1)
    e = K * E.exp(-r * T)
    return E.fnms(e, E.normcdf(d2), S * E.normcdf(d1)), E.fnms(S, E.normcdf(-d1), e * E.normcdf(-d2))


@pytest.mark.parametrize("n", [1, 3, 4, 1027, 1 << 18])
def test_blackscholes_compiled_kernel_reproduces_nt2(lib, dev, oracle, n):
    S, K, T = bs_inputs(n, seed=n)
    tS, tK, tT = (torch.from_numpy(a).to(dev) for a in (S, K, T))
    c, p = torch.empty_like(tS), torch.empty_like(tS)
    prog = E.assign([c, p], _bs_generic(E.Table(tS), E.Table(tK), E.Table(tT), E.Scalar(SIGMA), E.Scalar(R)),
                    precision=lib.PREC_NT2, force_generic=JIT)
    prog.jit_prepare(lib.PREC_NT2)
    torch.cuda.synchronize()
    rc, rp = oracle.blackscholes(S, K, T, R, SIGMA)
    assert _bits_equal(c.cpu().numpy(), rc) and _bits_equal(p.cpu().numpy(), rp)


def test_compiled_kernel_in_place_and_tie_forwarding(lib, dev, oracle):
    """sigma-delta through the compiled kernel: in-place tables, uint8 words,
    a later child reading a table an earlier child stored."""
    from helpers import sigmadelta_frames
    frames = sigmadelta_frames(h=64, w=77, frames=5, seed=3)
    F, H, W = frames.shape
    n = H * W
    rb, rv = frames[0].ravel().copy(), np.ones(n, np.uint8)
    tb, tv = torch.from_numpy(rb.copy()).to(dev), torch.from_numpy(rv.copy()).to(dev)
    tl = torch.zeros(n, dtype=torch.uint8, device=dev)
    for k in range(1, F):
        fr = torch.from_numpy(frames[k].ravel().copy()).to(dev)
        FR, B, V = E.Table(fr), E.Table(tb), E.Table(tv)
        nb = E.selinc(B < FR, E.seldec(B > FR, B))
        d = E.max_(B, FR) - E.min_(B, FR)
        m = E.adds(E.adds(d, d), d)
        nv = E.if_else(d.ne(0), E.selinc(V < m, E.seldec(V > m, V)), V)
        E.assign([tb, tv, tl], [nb, nv, E.if_zero_else_one(d < V, 1)], force_generic=JIT).jit_prepare(0)
        rb, rv, rl = oracle.sigmadelta(frames[k].ravel(), rb, rv)
        torch.cuda.synchronize()
        assert _bits_equal(tb.cpu().numpy(), rb) and _bits_equal(tv.cpu().numpy(), rv)
        assert _bits_equal(tl.cpu().numpy(), rl), k
