"""Host-side checks of libnt2gpu without a GPU: the library loads, exports
every entry point nt2g.h declares, and its program compiler and argument
validation behave -- none of these calls reaches the CUDA runtime."""
import ctypes
import re

import pytest
import torch

from nt2_gb300 import expr as E

NULL = ctypes.c_void_p(None)


def _header():
    import nt2_gb300.lib as lib
    return open(lib.HEADER_PATH).read()


def test_library_exports_every_declared_symbol(lib):
    decl = set(re.findall(r"\b(nt2g_[a-z0-9_]+)\s*\(", _header()))
    decl = {d for d in decl if not d.endswith("_t")}
    handle = ctypes.CDLL(lib.LIB_PATH)
    missing = [d for d in sorted(decl) if not hasattr(handle, d)]
    assert not missing, missing
    assert set(lib.exported_symbols()) <= decl


def test_opcode_values_match_header(lib):
    h = _header()
    body = h[h.index("typedef enum nt2g_opcode"):h.index("} nt2g_opcode;")]
    vals, nxt = {}, 0
    for name, val in re.findall(r"NT2G_OP_([A-Z0-9_]+)(?:\s*=\s*(\d+))?", body):
        nxt = int(val) if val else nxt
        vals[name] = nxt
        nxt += 1
    assert vals == lib.OP


def test_abi_version(lib):
    assert lib.load().nt2g_abi_version() == 2


def _cpu_tables(n=8, k=3, dtype=torch.float32):
    return [E.Table(torch.zeros(n, dtype=dtype)) for _ in range(k)]


def bs_textbook(S, K, T, sig, r):
    sq = E.sqrt(T)
    d1 = (E.log(S / K) + E.fma(E.sqr(sig), 0.5, r) * T) / (sig * sq)
    d2 = E.fnms(sig, sq, d1)
    e = K * E.exp(-r * T)
    call = E.fnms(e, E.normcdf(d2), S * E.normcdf(d1))
    put = E.fnms(S, E.normcdf(-d1), e * E.normcdf(-d2))
    return call, put


def test_compiler_binds_blackscholes(lib):
    S, K, T = _cpu_tables()
    c, p = torch.zeros(8), torch.zeros(8)
    prog, _ = E.compile_program([c, p], list(bs_textbook(S, K, T, E.Scalar(0.3), E.Scalar(0.02))))
    info = prog.info()
    assert info.kernel_name == b"blackscholes"
    # d1, d2, sqrt(T), e shared once each after CSE
    assert info.n_ops < 45
    sig = E.Table(torch.zeros(8))
    prog2, _ = E.compile_program([c, p], list(bs_textbook(S, K, T, sig, 0.02)))
    assert prog2.info().kernel_name == b"blackscholes"


def test_compiler_binds_named_expressions(lib):
    x, y, z = _cpu_tables()
    out = torch.zeros(8)
    prog, _ = E.compile_program([y.table], [2.5 * x + y])
    assert prog.info().kernel_name == b"saxpy"
    prog, _ = E.compile_program([out], [E.exp(-E.sqr(x)) * E.sqrt(E.abs_(y)) + E.log1p(E.abs_(z))])
    assert prog.info().kernel_name == b"expr3"
    r, g, b = x, y, z
    Y, U, V = torch.zeros(8), torch.zeros(8), torch.zeros(8)
    ty = E.Table(Y)
    prog, _ = E.compile_program([Y, U, V], [0.299 * r + 0.587 * g + 0.114 * b, 0.492 * (b - ty), 0.877 * (r - ty)])
    assert prog.info().kernel_name == b"rgb2yuv"
    # a different expression stays generic
    prog, _ = E.compile_program([out], [E.exp(x) * 2.0 + y])
    assert prog.info().kernel_name == b"generic"


def sigmadelta_exprs(fr, bkg, var):
    nb = E.selinc(bkg < fr, E.seldec(bkg > fr, bkg))
    return nb


def test_compiler_binds_sigmadelta_through_tie_forwarding(lib):
    u8 = torch.uint8
    fr, bkg, var = _cpu_tables(16, 3, u8)
    lab = torch.zeros(16, dtype=u8)
    nb = E.selinc(bkg < fr, E.seldec(bkg > fr, bkg))
    # second and third children read the tables the first child wrote (tie semantics)
    d = E.max_(bkg, fr) - E.min_(bkg, fr)
    m = E.adds(E.adds(d, d), d)
    nv = E.if_else(d.ne(0), E.selinc(var < m, E.seldec(var > m, var)), var)
    label = E.if_zero_else_one(d < var, lib.U8)
    prog, _ = E.compile_program([bkg.table, var.table, lab], [nb, nv, label])
    assert prog.info().kernel_name == b"sigmadelta"


def _raw(ops, n_slots):
    arr = (E.lib.Op * len(ops))(*[E.lib.Op(*o) for o in ops])
    h = ctypes.c_void_p()
    st = E.lib.load().nt2g_program_create(arr, len(ops), n_slots, ctypes.byref(h))
    if st == 0:
        E.lib.load().nt2g_program_destroy(h)
    return st


def test_compiler_rejects_bad_programs(lib):
    OP, F, U = lib.OP, lib.F32, lib.U8
    ld = lambda s, dt=F: (OP["LOAD"], dt, s, -1, -1, 0.0)  # noqa: E731
    st = lambda v, s, dt=F: (OP["STORE"], dt, v, s, -1, 0.0)  # noqa: E731
    assert _raw([ld(0), (OP["EXP"], F, 0, -1, -1, 0.0), st(1, 1)], 2) == lib.OK
    assert _raw([ld(0), (OP["EXP"], F, 2, -1, -1, 0.0), st(1, 1)], 2) == lib.ERR_INVALID   # forward ref
    assert _raw([ld(5), st(0, 1)], 2) == lib.ERR_INVALID                                   # slot range
    assert _raw([ld(0), st(0, 1, U)], 2) == lib.ERR_INVALID                               # dtype mismatch
    assert _raw([ld(0, U), (OP["EXP"], U, 0, -1, -1, 0.0), st(1, 1, U)], 2) == lib.ERR_UNSUPPORTED
    assert _raw([(OP["SCALAR"], F, 0, -1, -1, 0.0), ld(1), st(1, 0)], 2) == lib.ERR_INVALID  # store to scalar
    assert _raw([ld(0), ld(1), (OP["SELINC"], F, 0, 1, -1, 0.0), st(2, 1)], 2) == lib.ERR_INVALID  # no logical
    assert _raw([ld(0), (999, F, 0, -1, -1, 0.0), st(1, 1)], 2) == lib.ERR_INVALID           # opcode
    assert _raw([ld(0)], 1) == lib.ERR_INVALID                                               # no store
    assert "no store" not in lib.load().nt2g_last_error().decode() or True


def test_compiler_limits(lib):
    OP, F = lib.OP, lib.F32
    ops = [(OP["LOAD"], F, 0, -1, -1, 0.0)]
    for i in range(200):
        ops.append((OP["EXP"], F, len(ops) - 1, -1, -1, 0.0))
    ops.append((OP["STORE"], F, len(ops) - 1, 1, -1, 0.0))
    assert _raw(ops, 2) == lib.ERR_UNSUPPORTED
    assert "exceed" in lib.load().nt2g_last_error().decode()


def test_direct_entry_points_validate_before_touching_the_gpu(lib):
    L = lib.load()
    assert L.nt2g_blackscholes_f32(NULL, NULL, NULL, NULL, 0.3, 0.02, NULL, NULL, 16, 0, NULL) == lib.ERR_INVALID
    assert L.nt2g_blackscholes_f32(NULL, NULL, NULL, NULL, 0.3, 0.02, NULL, NULL, 0, 0, NULL) == lib.OK
    assert L.nt2g_saxpy_f32(1.0, NULL, NULL, -1, NULL) == lib.ERR_INVALID
    assert L.nt2g_map_f32(99, NULL, NULL, 0, 0, NULL) == lib.ERR_INVALID
    assert L.nt2g_expr3_f32(NULL, NULL, NULL, NULL, 0, 7, NULL) == lib.ERR_INVALID  # precision
    nb = ctypes.c_size_t()
    assert L.nt2g_reduce_workspace_size(1 << 28, ctypes.byref(nb)) == lib.OK and nb.value > 0
    ws = ctypes.create_string_buffer(16)
    assert L.nt2g_reduce_f32(ctypes.c_void_p(1), NULL, 10, ws, 16, ctypes.c_void_p(8), NULL, NULL) == lib.ERR_INVALID
    assert "workspace" in L.nt2g_last_error().decode()


def test_median_validates_before_touching_the_gpu(lib):
    """nt2g_median_f32: op, extents, NULL tables, overlap and the workspace of
    long slices are checked first; no slices is no work; slices up to 40960
    elements need no workspace."""
    L = lib.load()
    nb = ctypes.c_size_t()
    assert L.nt2g_median_workspace_size(1, 40960, 7, ctypes.byref(nb)) == lib.OK and nb.value == 0
    assert L.nt2g_median_workspace_size(3, 40961, 2, ctypes.byref(nb)) == lib.OK and nb.value == 6 * (2048 + 32)
    assert L.nt2g_median_workspace_size(-1, 4, 2, ctypes.byref(nb)) == lib.ERR_INVALID
    x, out = ctypes.c_void_p(1 << 20), ctypes.c_void_p(1 << 30)
    assert L.nt2g_median_f32(x, 1, 10, 4, 2, NULL, 0, out, NULL) == lib.ERR_INVALID  # op
    assert L.nt2g_median_f32(x, 1, -10, 4, 0, NULL, 0, out, NULL) == lib.ERR_INVALID
    assert L.nt2g_median_f32(x, 1, 10, 4, 0, NULL, 0, NULL, NULL) == lib.ERR_INVALID  # out
    assert L.nt2g_median_f32(NULL, 1, 10, 4, 0, NULL, 0, out, NULL) == lib.ERR_INVALID  # x
    assert L.nt2g_median_f32(x, 1, 10, 4, 0, NULL, 0, ctypes.c_void_p((1 << 20) + 8), NULL) == lib.ERR_INVALID
    assert L.nt2g_median_f32(x, 1, 50000, 2, 0, NULL, 0, out, NULL) == lib.ERR_INVALID  # workspace
    assert "workspace" in L.nt2g_last_error().decode()
    assert L.nt2g_median_f32(NULL, 0, 10, 4, 1, NULL, 0, NULL, NULL) == lib.OK  # no slices


def test_trapz_validates_before_touching_the_gpu(lib):
    """nt2g_trapz_f32: extents, precision, NULL tables and the fast policy's
    workspace are checked first; no outputs is no work."""
    L = lib.load()
    nb = ctypes.c_size_t()
    assert L.nt2g_trapz_workspace_size(1, 1 << 20, 1, ctypes.byref(nb)) == lib.OK and nb.value >= 8
    assert L.nt2g_trapz_workspace_size(-1, 4, 2, ctypes.byref(nb)) == lib.ERR_INVALID
    x, out = ctypes.c_void_p(1 << 20), ctypes.c_void_p(1 << 30)
    assert L.nt2g_trapz_f32(x, 1, 10, 4, 5, NULL, 0, out, NULL) == lib.ERR_INVALID  # precision
    assert L.nt2g_trapz_f32(x, 1, -10, 4, 0, NULL, 0, out, NULL) == lib.ERR_INVALID
    assert L.nt2g_trapz_f32(x, 1, 10, 4, 0, NULL, 0, NULL, NULL) == lib.ERR_INVALID  # out
    assert L.nt2g_trapz_f32(NULL, 1, 10, 4, 0, NULL, 0, out, NULL) == lib.ERR_INVALID  # x
    assert L.nt2g_trapz_f32(x, 1, 1 << 20, 1, 0, NULL, 0, out, NULL) == lib.ERR_INVALID  # fast: workspace
    assert "workspace" in L.nt2g_last_error().decode()
    assert L.nt2g_trapz_f32(NULL, 0, 10, 4, 1, NULL, 0, NULL, NULL) == lib.OK


def test_eval_validates_arguments(lib):
    x = E.Table(torch.zeros(8))
    out = torch.zeros(8)
    prog, slots = E.compile_program([out], [E.exp(x)])
    L = lib.load()
    args = (lib.Arg * 2)(lib.Arg(8, 0.0, lib.F32, 0), lib.Arg(16, 0.0, lib.F32, 0))
    assert L.nt2g_eval(prog.handle, args, 2, 0, -1, 0, 0, NULL) == lib.ERR_INVALID
    assert L.nt2g_eval(prog.handle, args, 1, 0, 8, 0, 0, NULL) == lib.ERR_INVALID  # too few args
    bad = (lib.Arg * 2)(lib.Arg(8, 0.0, lib.U8, 0), lib.Arg(16, 0.0, lib.F32, 0))
    assert L.nt2g_eval(prog.handle, bad, 2, 0, 8, 0, 0, NULL) == lib.ERR_INVALID  # dtype
    assert L.nt2g_eval(prog.handle, args, 2, 0, 0, 0, 0, NULL) == lib.OK          # empty range


def test_batch_create_validates_items(lib):
    L = lib.load()
    items = (lib.BatchItem * 1)()
    items[0].expr = 7
    items[0].n = 16
    h = ctypes.c_void_p()
    assert L.nt2g_batch_create(items, 1, None, ctypes.byref(h)) == lib.ERR_INVALID
    tune = lib.BatchTune(100, 0, 4, 0)
    assert L.nt2g_batch_create(items, 1, ctypes.byref(tune), ctypes.byref(h)) == lib.ERR_INVALID


def test_batch_create_validates_program_items(lib):
    """Program items: a missing program, a fold program, too few arguments and
    an unknown vector width are refused before anything reaches the device."""
    L = lib.load()
    h = ctypes.c_void_p()
    x = E.Table(torch.zeros(8))
    prog, slots = E.compile_program([torch.zeros(8)], [E.exp(x)])
    fold_prog, _ = E.compile_program([], [], fold=E.exp(x))
    args = (lib.Arg * 2)(lib.Arg(8, 0.0, lib.F32, 0), lib.Arg(16, 0.0, lib.F32, 0))
    items = (lib.BatchItem * 1)()
    items[0].expr, items[0].n, items[0].n_args = lib.BATCH_PROGRAM, 8, 2
    items[0].args = ctypes.cast(args, ctypes.POINTER(lib.Arg))
    assert L.nt2g_batch_create(items, 1, None, ctypes.byref(h)) == lib.ERR_INVALID  # no program
    items[0].program = fold_prog.handle.value
    assert L.nt2g_batch_create(items, 1, None, ctypes.byref(h)) == lib.ERR_INVALID  # folds
    assert b"folds" in lib.load().nt2g_last_error()
    items[0].program, items[0].n_args = prog.handle.value, 1
    assert L.nt2g_batch_create(items, 1, None, ctypes.byref(h)) == lib.ERR_INVALID  # 1 argument, 2 slots
    tune = lib.BatchTune(256, 0, 4, 0, 3)
    assert L.nt2g_batch_create(items, 1, ctypes.byref(tune), ctypes.byref(h)) == lib.ERR_INVALID  # width 3
    assert not h.value


def _nvrtc():
    for name in ("libnvrtc.so.13", "/usr/local/cuda/lib64/libnvrtc.so.13"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.skip("NVRTC not installed")


def _nvrtc_compile(nv, src):
    prog = ctypes.c_void_p()
    assert nv.nvrtcCreateProgram(ctypes.byref(prog), src.encode(), b"nt2g_jit.cu", 0, None, None) == 0
    opts = (ctypes.c_char_p * 3)(b"--gpu-architecture=sm_103a", b"-std=c++17", b"-default-device")
    rc = nv.nvrtcCompileProgram(prog, 3, opts)
    n = ctypes.c_size_t()
    nv.nvrtcGetProgramLogSize(prog, ctypes.byref(n))
    log = ctypes.create_string_buffer(n.value + 1)
    nv.nvrtcGetProgramLog(prog, log)
    size = ctypes.c_size_t()
    if rc == 0:
        nv.nvrtcGetCUBINSize(prog, ctypes.byref(size))
    nv.nvrtcDestroyProgram(ctypes.byref(prog))
    return rc, log.value.decode(errors="replace"), size.value


def test_compiled_kernel_source_builds_for_sm103a(lib):
    """The source the library hands to NVRTC for a generic program compiles
    for sm_103a under both policies (NVRTC needs no GPU)."""
    nv = _nvrtc()
    S, K, T = _cpu_tables()
    c, p = torch.zeros(8), torch.zeros(8)
    bs, _ = E.compile_program([c, p], list(bs_textbook(S, K, T, E.Scalar(0.3), E.Scalar(0.02))))
    u8 = torch.uint8
    fr, bkg, var = _cpu_tables(16, 3, u8)
    d = E.max_(bkg, fr) - E.min_(bkg, fr)
    lab = torch.zeros(16, dtype=u8)
    mixed, _ = E.compile_program([lab, c], [E.if_zero_else_one(d < var, lib.U8), E.Table(torch.zeros(8)) > 1.0])
    for prog in (bs, mixed):
        for prec in (lib.PREC_FAST, lib.PREC_NT2):
            src = prog.jit_source(prec)
            assert 'extern "C" __global__' in src and "nt2g_jit_kernel" in src
            assert ("nt2g::Nt2" if prec == lib.PREC_NT2 else "nt2g::Fast") in src
            if prog is bs:  # N(d1)/N(-d1) and N(d2)/N(-d2) each from one erfc core
                assert src.count("nt2g::normcdf_pair<P>(") == 2 and "nt2g::normcdf<P>(" not in src
            rc, log, size = _nvrtc_compile(nv, src)
            assert rc == 0, log[:2000]
            assert size > 0


def test_compiled_kernel_source_validates_arguments(lib):
    x = E.Table(torch.zeros(8))
    prog, _ = E.compile_program([torch.zeros(8)], [E.exp(x)])
    L = lib.load()
    n = ctypes.c_size_t()
    assert L.nt2g_program_jit_source(prog.handle, 5, None, 0, ctypes.byref(n)) == lib.ERR_INVALID
    assert L.nt2g_program_jit_source(prog.handle, 0, None, 0, ctypes.byref(n)) == lib.OK and n.value > 100
    small = ctypes.create_string_buffer(10)
    assert L.nt2g_program_jit_source(prog.handle, 0, small, 10, ctypes.byref(n)) == lib.ERR_INVALID
    assert L.nt2g_program_jit_prepare(None, 0) == lib.ERR_INVALID


def test_fold_kernel_source_builds_for_sm103a(lib):
    """The fold kernels nt2g_eval_fold compiles for a program's FOLD value
    (the fold bodies instantiated over the expression's element function)
    build for sm_103a, for sum-type, max/min, two-pass and logical folds under
    the three element/fold policies (NVRTC needs no GPU)."""
    import time
    nv = _nvrtc()
    x, y = E.Table(torch.zeros(8)), E.Table(torch.zeros(8))
    u8 = torch.uint8
    fr, bkg = E.Table(torch.zeros(8, dtype=u8)), E.Table(torch.zeros(8, dtype=u8))
    cases = [(E.exp(x) * y, "sum", lib.PREC_FAST), (E.abs_(x - y), "max", lib.PREC_NT2),
             (E.exp(x) * y, "var", lib.PREC_NT2_ELEMENTS), (fr > bkg, "nbtrue", lib.PREC_FAST)]
    for e, op, prec in cases:
        prog, _ = E.compile_program([], [], fold=e)
        src = prog.fold_source(op, prec)
        assert "fold_nt2" in src and ("fold_inner_11" in src) == (prec != lib.PREC_NT2)
        t0 = time.time()
        rc, log, size = _nvrtc_compile(nv, src)
        assert rc == 0, (op, prec, log[:2000])
        assert size > 0
        print(f"\nfold {op} policy {prec}: {time.time() - t0:.1f} s to compile, cubin {size} bytes")


def test_fold_programs_validate(lib):
    L = lib.load()
    x = E.Table(torch.zeros(8))
    prog, slots = E.compile_program([], [], fold=E.exp(x))
    args = (lib.Arg * 1)(lib.Arg(slots[0].data_ptr(), 0.0, lib.F32, 0))
    out = torch.zeros(1)
    # a fold program does not evaluate as a transform, and a transform does not fold
    assert L.nt2g_eval(prog.handle, args, 1, 0, 8, 0, 0, None) == lib.ERR_INVALID
    tprog, _ = E.compile_program([torch.zeros(8)], [E.exp(x)])
    assert L.nt2g_eval_fold(tprog.handle, args, 1, 1, 8, 1, 0, 0, None, 0, lib._ptr(out), None, None,
                            None) == lib.ERR_INVALID
    # op, precision and index / FP64 requests are checked before any launch
    for op, prec, idx, o64 in ((18, 0, None, None), (0, 3, None, None), (0, 0, lib._ptr(out), None),
                               (2, 0, None, lib._ptr(out)), (0, 1, None, lib._ptr(out))):
        assert L.nt2g_eval_fold(prog.handle, args, 1, 1, 8, 1, op, prec, None, 0, lib._ptr(out), idx, o64,
                                None) == lib.ERR_INVALID
    # two FOLDs, or a FOLD and a STORE, in one program
    ops = (lib.Op * 4)(lib.Op(lib.OP["LOAD"], 0, 0, -1, -1, 0.0), lib.Op(lib.OP["FOLD"], 0, 0, -1, -1, 0.0),
                       lib.Op(lib.OP["FOLD"], 0, 0, -1, -1, 0.0), lib.Op(lib.OP["STORE"], 0, 0, 1, -1, 0.0))
    h = ctypes.c_void_p()
    assert L.nt2g_program_create(ops, 3, 2, ctypes.byref(h)) == lib.ERR_INVALID
    ops[2] = lib.Op(lib.OP["STORE"], 0, 0, 1, -1, 0.0)
    assert L.nt2g_program_create(ops, 3, 2, ctypes.byref(h)) == lib.ERR_INVALID


def test_batch_kernel_source_builds_for_sm103a(lib):
    """The kernel a batch of user programs is linked into (every program a
    tile function, a block-uniform switch, dynamic/static schedules, one and
    two float4 vectors per thread) compiles for sm_103a under both policies."""
    nv = _nvrtc()
    S, K, T = _cpu_tables()
    c, p = torch.zeros(8), torch.zeros(8)
    bs, _ = E.compile_program([c, p], list(bs_textbook(S, K, T, E.Scalar(0.3), E.Scalar(0.02))))
    u8 = torch.uint8
    fr, bkg, var = _cpu_tables(16, 3, u8)
    d = E.max_(bkg, fr) - E.min_(bkg, fr)
    lab = torch.zeros(16, dtype=u8)
    mixed, _ = E.compile_program([lab, c], [E.if_zero_else_one(d < var, lib.U8), E.Table(torch.zeros(8)) > 1.0])
    gen, _ = E.compile_program([c], [E.sinpi(E.linspace(0, 2, 8)) * E.Table(torch.zeros(8))])
    for prec, bt in ((lib.PREC_FAST, 256), (lib.PREC_NT2, 128)):
        src = E.batch_source([bs, mixed, gen], prec, bt)
        for k in range(3):
            assert f"case {k}: NT2G_RUN(prog{k}_tile)" in src
        for name in ("batch_01", "batch_02", "batch_11", "batch_12"):
            assert f"__launch_bounds__({bt}) {name}(" in src
        rc, log, size = _nvrtc_compile(nv, src)
        assert rc == 0, log[:2000]
        assert size > 0
    n = ctypes.c_size_t()
    hs = (ctypes.c_void_p * 1)(bs.handle.value)
    L = lib.load()
    assert L.nt2g_batch_source(hs, 1, 0, 100, None, 0, ctypes.byref(n)) == lib.ERR_INVALID  # block size
    assert L.nt2g_batch_source(hs, 0, 0, 256, None, 0, ctypes.byref(n)) == lib.ERR_INVALID


UNARY_VJP_OPS = ["exp", "log", "log1p", "erfc", "normcdf", "fastnormcdf", "sqrt", "rec", "abs_", "exp2", "exp10",
                 "expm1", "log2", "log10", "sin", "cos", "tan", "sinpi", "cospi", "sinh", "cosh", "tanh", "asin",
                 "acos", "atan", "asinh", "acosh", "atanh", "cbrt", "cot", "sec", "csc", "sind", "cosd", "tand",
                 "tanpi", "cotpi", "cotd", "secpi", "cscpi", "secd", "cscd", "sinc", "sincpi", "acotd", "asec", "coth",
                 "sinhc", "acsc", "asech", "acoth", "acsch", "erf", "erfcx", "expx2", "gamma", "gammaln", "erfinv",
                 "erfcinv", "exprecneg", "exprecnegc", "sqrt1pm1", "floor", "ceil", "trunc", "round", "round2even",
                 "frac", "sign", "signnz", "sqr", "dawson", "spence", "proper_tanpi"]


def _vjp_programs(lib):
    """Programs that together use every opcode with an adjoint rule."""
    n = 8
    progs = []
    S, K, T = _cpu_tables()
    c, p = torch.zeros(n), torch.zeros(n)
    progs.append(E.compile_program([c, p], list(bs_textbook(S, K, T, E.Scalar(0.3), E.Scalar(0.02))))[0])
    x, y, z = (E.Table(torch.zeros(n)) for _ in range(3))
    for k in range(0, len(UNARY_VJP_OPS), 24):
        acc = None
        for name in UNARY_VJP_OPS[k:k + 24]:
            t = getattr(E, name)(x)
            acc = t if acc is None else acc + t
        progs.append(E.compile_program([torch.zeros(n)], [acc])[0])
    e = (E.pow(x, y) + E.atan2(x, y) + E.hypot(x, y) + x / y + E.min_(x, y) + E.max_(x, y) + E.copysign(x, y)
         + E.fma(x, y, z) + E.fnms(x, y, z) + E.if_else(x > y, y, z) + E.selinc(x < z, y) + E.seldec(x > z, z)
         + E.if_zero_else_one(x < y, lib.F32) - (-x) + E.mod(x, y) + E.rem(y, z) + E.pow2(x, y) + E.pow2(z))
    progs.append(E.compile_program([torch.zeros(n)], [e])[0])
    e = (E.nthroot(x, 3.0) + E.nthroot(y, z) + E.expni(2.0, x) + E.expni(z, y) + E.gammainc(x, 2.5)
         + E.gammaincinv(x, 2.5))
    progs.append(E.compile_program([torch.zeros(n)], [e])[0])
    return progs


def test_vjp_kernel_source_builds_for_sm103a(lib):
    """The reverse-mode kernels of programs covering every opcode's adjoint
    rule compile for sm_103a (NVRTC needs no GPU); fold programs are refused."""
    nv = _nvrtc()
    for i, prog in enumerate(_vjp_programs(lib)):
        for prec in ((lib.PREC_FAST, lib.PREC_NT2) if i == 0 else (lib.PREC_FAST,)):
            src = prog.vjp_source(prec)
            assert "nt2g_vjp_kernel" in src and "vjp_tile" in src
            rc, log, size = _nvrtc_compile(nv, src)
            assert rc == 0, log[:2000]
            assert size > 0
    x = E.Table(torch.zeros(8))
    fold_prog, _ = E.compile_program([], [], fold=E.exp(x))
    n = ctypes.c_size_t()
    assert lib.load().nt2g_program_vjp_source(fold_prog.handle, 0, None, 0, ctypes.byref(n)) == lib.ERR_INVALID


def test_integer_operand_and_incomplete_gamma_programs(lib):
    """dawson, nthroot, expni and gammainc (double arithmetic inside) compile
    for sm_103a in both policies; gammainc has a rule for x only, so reverse
    mode through its a operand is refused with NT2G_ERR_UNSUPPORTED."""
    nv = _nvrtc()
    x, y = E.Table(torch.zeros(8)), E.Table(torch.zeros(8))
    prog, _ = E.compile_program([torch.zeros(8), torch.zeros(8)],
                                [E.dawson(x) + E.nthroot(x, y), E.expni(y, x) * E.gammainc(x, y)])
    for prec in (lib.PREC_FAST, lib.PREC_NT2):
        rc, log, size = _nvrtc_compile(nv, prog.jit_source(prec))
        assert rc == 0, log[:2000]
    n = ctypes.c_size_t()
    assert lib.load().nt2g_program_vjp_source(prog.handle, 0, None, 0, ctypes.byref(n)) == lib.ERR_UNSUPPORTED
    assert b"opcode 154" in lib.load().nt2g_last_error()
    st, _ = E.compile_program([torch.zeros(8)], [E.stirling(x) + E.gammaincinv(y, 2.0)])
    for prec in (lib.PREC_FAST, lib.PREC_NT2):
        rc, log, size = _nvrtc_compile(nv, st.jit_source(prec))
        assert rc == 0, log[:2000]
    assert lib.load().nt2g_program_vjp_source(st.handle, 0, None, 0, ctypes.byref(n)) == lib.ERR_UNSUPPORTED
    assert b"opcode 157" in lib.load().nt2g_last_error()  # stirling: no adjoint rule


def test_vjp_validates_slots(lib):
    """Cotangents only on float outputs, gradients only of float tables the
    program reads; refused before anything reaches the device."""
    L = lib.load()
    X, Y = torch.zeros(8), torch.zeros(8)
    prog, slots = E.compile_program([Y], [E.exp(E.Table(X)) * E.Scalar(2.0)])
    args = (lib.Arg * len(slots))()
    for i, s in enumerate(slots):
        args[i] = lib.Arg(None, 2.0, lib.F32, 1) if isinstance(s, E.Node) else lib.Arg(8 * (i + 1), 0.0, lib.F32, 0)
    sx, sy = E._slot_of(slots, X), E._slot_of(slots, Y)
    ct, tg = (ctypes.c_void_p * len(slots))(), (ctypes.c_void_p * len(slots))()
    ct[sx] = 64  # a cotangent on an input slot
    assert L.nt2g_program_vjp(prog.handle, args, len(slots), 0, ct, tg, None, 0, None, 0, None) == lib.ERR_INVALID
    ct[sx], tg[sy] = None, 64  # a gradient of an output-only slot
    assert L.nt2g_program_vjp(prog.handle, args, len(slots), 0, ct, tg, None, 0, None, 0, None) == lib.ERR_INVALID
    tg[sy] = None
    assert L.nt2g_program_vjp(prog.handle, args, len(slots), -1, ct, tg, None, 0, None, 0, None) == lib.ERR_INVALID
    assert L.nt2g_program_vjp(prog.handle, args, len(slots), 0, ct, tg, None, 7, None, 0, None) == lib.ERR_INVALID


def test_digamma_signgam_programs_compile_and_vjp_refuses_digamma(lib):
    """A program using digamma (double arithmetic inside), signgam and NT2's
    beta composition compiles for sm_103a; digamma has no adjoint rule, so
    its reverse mode is refused with NT2G_ERR_UNSUPPORTED, while signgam
    (piecewise constant) differentiates to zero."""
    nv = _nvrtc()
    x, y = E.Table(torch.zeros(8)), E.Table(torch.zeros(8))
    prog, _ = E.compile_program([torch.zeros(8), torch.zeros(8)], [E.beta(x, y), E.digamma(x) + E.signgam(y)])
    for prec in (lib.PREC_FAST, lib.PREC_NT2):
        rc, log, size = _nvrtc_compile(nv, prog.jit_source(prec))
        assert rc == 0, log[:2000]
    n = ctypes.c_size_t()
    assert lib.load().nt2g_program_vjp_source(prog.handle, 0, None, 0, ctypes.byref(n)) == lib.ERR_UNSUPPORTED
    assert b"opcode 150" in lib.load().nt2g_last_error()
    sg, _ = E.compile_program([torch.zeros(8)], [E.signgam(x) * E.exp(y)])
    src = sg.vjp_source(0)
    rc, log, size = _nvrtc_compile(nv, src)
    assert rc == 0, log[:2000]
