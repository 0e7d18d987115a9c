"""ctypes binding of libnt2gpu (the C ABI declared in include/nt2g.h).

The library is built in-tree (nt2_gb300/_build/libnt2gpu.so) by
``nt2_gb300.build.build_library``.  Loading fails loudly when it is missing:
there is no CPU fallback for any entry point.

Tensors passed to the helpers here are CUDA torch tensors; only their data
pointers and the current stream cross the ABI.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libnt2gpu.so")
HEADER_PATH = os.path.join(os.path.dirname(_HERE), "include", "nt2g.h")

OK, ERR_INVALID, ERR_UNSUPPORTED, ERR_CUDA, ERR_DEVICE_FLAG, ERR_NOMEM = range(6)
PREC_FAST, PREC_NT2, PREC_NT2_ELEMENTS = 0, 1, 2
F32, U8 = 0, 1

# opcodes (values fixed by nt2g.h; tests check they agree with the header)
OP = dict(
    LOAD=1, SCALAR=2, CONST=3, STORE=4, INDEX=5, FOLD=6,
    ADD=10, SUB=11, MUL=12, DIV=13, NEG=14, ABS=15, SQR=16, SQRT=17, REC=18, MIN=19, MAX=20,
    FMA=30, FNMS=31,
    EXP=40, LOG=41, LOG1P=42, ERFC=43, NORMCDF=44, FASTNORMCDF=45, EXP2=46, EXP10=47, EXPM1=48, LOG2=49, LOG10=50,
    SIN=51, COS=52, TAN=53, SINPI=54, COSPI=55, POW=56, SINH=57, COSH=58, TANH=59,
    LT=60, GT=61, LE=62, GE=63, EQ=64, NE=65,
    IF_ELSE=70, SELINC=71, SELDEC=72, IF_ZERO_ELSE_ONE=73, ADDS=74,
    ASIN=90, ACOS=91, ATAN=92, ATAN2=93, ASINH=94, ACOSH=95, ATANH=96, CBRT=97, HYPOT=98,
    COT=100, SEC=101, CSC=102, SIND=103, COSD=104, TAND=105,
    TANPI=106, COTPI=107, COTD=108, SECPI=109, CSCPI=110, SECD=111, CSCD=112, SINC=113, SINCPI=114, ACOTD=115, ASEC=116, COTH=117, SINHC=118, ACSC=119, ASECH=120, ACOTH=121, ACSCH=122,
    ERF=123, ERFCX=124, EXPX2=125, GAMMA=126, GAMMALN=127, EXPRECNEG=128, EXPRECNEGC=129, SQRT1PM1=130, ERFINV=131, ERFCINV=132, SIGNGAM=149, DIGAMMA=150, DAWSON=151, NTHROOT=152, EXPNI=153, GAMMAINC=154, SPENCE=155, GAMMAINCINV=156, STIRLING=157, PROPER_TANPI=158, MOD=159, REM=160, POW2=161,
    FLOOR=133, CEIL=134, TRUNC=135, ROUND=136, ROUND2EVEN=137, FRAC=138, SIGN=139, SIGNNZ=140, COPYSIGN=141,
    IS_NAN=142, IS_INF=143, IS_FINITE=144, IS_EQZ=145, IS_NEZ=146, IS_LTZ=147, IS_GTZ=148,
)

MAP_FN = dict(exp=0, log=1, log1p=2, erfc=3, normcdf=4, fastnormcdf=5, sqrt=6, normcdf_neg=7, exp2=8, exp10=9,
              expm1=10, log2=11, log10=12, sin=13, cos=14, tan=15, sinpi=16, cospi=17,
              sinh=18, cosh=19, tanh=20, asin=21, acos=22, atan=23, asinh=24, acosh=25, atanh=26, cbrt=27,
              cot=28, sec=29, csc=30, sind=31, cosd=32, tand=33,
              tanpi=34, cotpi=35, cotd=36, secpi=37, cscpi=38, secd=39, cscd=40, sinc=41, sincpi=42, acotd=43, asec=44, coth=45, sinhc=46, acsc=47, asech=48, acoth=49, acsch=50,
              erf=64, erfcx=65, expx2=66, gamma=67, gammaln=68, erfinv=69, erfcinv=70, digamma=71, signgam=72, dawson=73, spence=74, stirling=75, exprecneg=80, exprecnegc=81, sqrt1pm1=82)

BATCH_BLACKSCHOLES, BATCH_SAXPY, BATCH_EXPR3, BATCH_PROGRAM = 0, 1, 2, 3


class Op(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int16), ("dtype", ctypes.c_int16), ("a", ctypes.c_int32),
                ("b", ctypes.c_int32), ("c", ctypes.c_int32), ("imm", ctypes.c_float)]


class Arg(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("scalar", ctypes.c_double), ("dtype", ctypes.c_int32),
                ("kind", ctypes.c_int32)]


class ProgramInfo(ctypes.Structure):
    _fields_ = [("kernel", ctypes.c_int32), ("n_ops", ctypes.c_int32), ("n_regs", ctypes.c_int32),
                ("n_slots", ctypes.c_int32), ("kernel_name", ctypes.c_char * 48)]


class BatchItem(ctypes.Structure):
    _fields_ = [("expr", ctypes.c_int32), ("n_args", ctypes.c_int32), ("n", ctypes.c_int64),
                ("inp", ctypes.c_void_p * 3), ("out", ctypes.c_void_p * 2), ("s", ctypes.c_float * 2),
                ("program", ctypes.c_void_p), ("args", ctypes.POINTER(Arg))]


class BatchTune(ctypes.Structure):
    _fields_ = [("block_threads", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32),
                ("tile_vectors", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("vector_width", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Nt2gError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"nt2g status {status}: {message}")
        self.status = status


_VP, _I64, _I32, _F, _D = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_float, ctypes.c_double
_SIGNATURES = {
    "nt2g_last_error": (ctypes.c_char_p, []),
    "nt2g_abi_version": (ctypes.c_int, []),
    "nt2g_program_create": (_I32, [ctypes.POINTER(Op), _I32, _I32, ctypes.POINTER(_VP)]),
    "nt2g_program_info_get": (_I32, [_VP, ctypes.POINTER(ProgramInfo)]),
    "nt2g_program_destroy": (None, [_VP]),
    "nt2g_eval": (_I32, [_VP, ctypes.POINTER(Arg), _I32, _I64, _I64, _I32, _I32, _VP]),
    "nt2g_program_jit_source": (_I32, [_VP, _I32, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "nt2g_program_jit_prepare": (_I32, [_VP, _I32]),
    "nt2g_blackscholes_f32": (_I32, [_VP, _VP, _VP, _VP, _F, _F, _VP, _VP, _I64, _I32, _VP]),
    "nt2g_blackscholes_demo_f32": (_I32, [_VP, _VP, _VP, _VP, _F, _VP, _F, _VP, _I64, _I32, _VP]),
    "nt2g_blackscholes_vjp_f32": (_I32, [_VP, _VP, _VP, _VP, _F, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                                         _I64, _VP]),
    "nt2g_saxpy_f32": (_I32, [_F, _VP, _VP, _I64, _VP]),
    "nt2g_expr3_f32": (_I32, [_VP, _VP, _VP, _VP, _I64, _I32, _VP]),
    "nt2g_rgb2yuv_f32": (_I32, [_VP, _VP, _VP, _VP, _VP, _VP, _I64, _I32, _VP]),
    "nt2g_sigmadelta_u8": (_I32, [_VP, _VP, _VP, _VP, _I64, _VP]),
    "nt2g_sigmadelta_frames_u8": (_I32, [_VP, _VP, _VP, _VP, _I64, _I32, _VP]),
    "nt2g_map_f32": (_I32, [_I32, _VP, _VP, _I64, _I32, _VP]),
    "nt2g_reduce_workspace_size": (_I32, [_I64, ctypes.POINTER(ctypes.c_size_t)]),
    "nt2g_reduce_f32": (_I32, [_VP, _VP, _I64, _VP, ctypes.c_size_t, _VP, _VP, _VP]),
    "nt2g_reduce_f32_noalloc": (_I32, [_VP, _VP, _I64, _VP, _VP, _VP]),
    "nt2g_batch_create": (_I32, [ctypes.POINTER(BatchItem), _I32, ctypes.POINTER(BatchTune), ctypes.POINTER(_VP)]),
    "nt2g_batch_destroy": (None, [_VP]),
    "nt2g_batch_run": (_I32, [_VP, _VP]),
    "nt2g_batch_run_per_table": (_I32, [_VP, _VP]),
    "nt2g_batch_run_graph": (_I32, [_VP, _VP]),
    "nt2g_batch_source": (_I32, [ctypes.POINTER(_VP), _I32, _I32, _I32, ctypes.c_char_p, ctypes.c_size_t,
                                  ctypes.POINTER(ctypes.c_size_t)]),
    "nt2g_batch_autotune": (_I32, [ctypes.POINTER(BatchItem), _I32, ctypes.POINTER(BatchTune), _I32, _I32, _I32, _VP,
                                    ctypes.POINTER(BatchTune), ctypes.POINTER(ctypes.c_float)]),
    "nt2g_batch_stats": (_I32, [_VP, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "nt2g_host_access": (_I32, [ctypes.POINTER(_I32)]),
    "nt2g_fold_workspace_size": (_I32, [_I64, _I64, _I64, ctypes.POINTER(ctypes.c_size_t)]),
    "nt2g_fold_f32": (_I32, [_VP, _I64, _I64, _I64, _I32, _I32, _VP, ctypes.c_size_t, _VP, _VP, _VP]),
    "nt2g_median_workspace_size": (_I32, [_I64, _I64, _I64, ctypes.POINTER(ctypes.c_size_t)]),
    "nt2g_trapz_workspace_size": (_I32, [_I64, _I64, _I64, ctypes.POINTER(ctypes.c_size_t)]),
    "nt2g_trapz_f32": (_I32, [_VP, _I64, _I64, _I64, _I32, _VP, ctypes.c_size_t, _VP, _VP]),
    "nt2g_median_f32": (_I32, [_VP, _I64, _I64, _I64, _I32, _VP, ctypes.c_size_t, _VP, _VP]),
    "nt2g_wait_timeouts": (_I32, [ctypes.POINTER(ctypes.c_uint64)]),
    "nt2g_program_vjp": (_I32, [_VP, ctypes.POINTER(Arg), _I32, _I64, ctypes.POINTER(_VP), ctypes.POINTER(_VP), _VP,
                                _I32, _VP, ctypes.c_size_t, _VP]),
    "nt2g_program_vjp_workspace_size": (_I32, [_VP, _I64, ctypes.POINTER(ctypes.c_size_t)]),
    "nt2g_program_vjp_source": (_I32, [_VP, _I32, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "nt2g_eval_fold": (_I32, [_VP, ctypes.POINTER(Arg), _I32, _I64, _I64, _I64, _I32, _I32, _VP, ctypes.c_size_t, _VP,
                              _VP, _VP, _VP]),
    "nt2g_program_fold_source": (_I32, [_VP, _I32, _I32, ctypes.c_char_p, ctypes.c_size_t,
                                        ctypes.POINTER(ctypes.c_size_t)]),
    "nt2g_scan_workspace_size": (_I32, [_I64, _I64, _I64, ctypes.POINTER(ctypes.c_size_t)]),
    "nt2g_scan_f32": (_I32, [_VP, _I64, _I64, _I64, _I32, _I32, _VP, ctypes.c_size_t, _VP, _VP]),
    "nt2g_device_alloc": (_I32, [ctypes.c_size_t, ctypes.POINTER(_VP)]),
    "nt2g_device_free": (_I32, [_VP]),
    "nt2g_memcpy": (_I32, [_VP, _VP, ctypes.c_size_t, _I32, _VP]),
    "nt2g_stream_synchronize": (_I32, [_VP]),
    "nt2g_device_current": (_I32, [ctypes.POINTER(_I32)]),
    "nt2g_stream_create": (_I32, [ctypes.POINTER(_VP)]),
    "nt2g_stream_destroy": (_I32, [_VP]),
}

_lib = None


def load():
    """Load libnt2gpu.so (once).  Raises if the library has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libnt2gpu is not built ({LIB_PATH} missing); run __graft_entry__.build()")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def exported_symbols():
    return list(_SIGNATURES)


def check(status):
    if status != OK:
        raise Nt2gError(status, load().nt2g_last_error().decode())


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


# ----------------------------------------------------------- direct kernels
def blackscholes(S, K, T, call, put, r, sigma=None, sigma_s=0.0, precision=PREC_FAST, stream=None):
    check(load().nt2g_blackscholes_f32(_ptr(S), _ptr(K), _ptr(T), _ptr(sigma), sigma_s, r, _ptr(call), _ptr(put),
                                       S.numel(), precision, _stream(stream)))


def blackscholes_demo(S, X, T, R, r=0.0, v=0.0, r_t=None, v_t=None, precision=PREC_FAST, stream=None):
    check(load().nt2g_blackscholes_demo_f32(_ptr(S), _ptr(X), _ptr(T), _ptr(r_t), r, _ptr(v_t), v, _ptr(R),
                                            S.numel(), precision, _stream(stream)))


def blackscholes_vjp(S, K, T, sigma, r, gc, gp, outs, stream=None):
    """outs: (call, put, dS, dK, dT, dsigma, dr) preallocated tensors."""
    check(load().nt2g_blackscholes_vjp_f32(_ptr(S), _ptr(K), _ptr(T), _ptr(sigma), r, _ptr(gc), _ptr(gp),
                                           *[_ptr(o) for o in outs], S.numel(), _stream(stream)))


def saxpy(alpha, X, Y, stream=None):
    check(load().nt2g_saxpy_f32(alpha, _ptr(X), _ptr(Y), X.numel(), _stream(stream)))


def expr3(x, y, z, out, precision=PREC_FAST, stream=None):
    check(load().nt2g_expr3_f32(_ptr(x), _ptr(y), _ptr(z), _ptr(out), x.numel(), precision, _stream(stream)))


def rgb2yuv(r, g, b, y, u, v, precision=PREC_FAST, stream=None):
    check(load().nt2g_rgb2yuv_f32(_ptr(r), _ptr(g), _ptr(b), _ptr(y), _ptr(u), _ptr(v), r.numel(), precision,
                                  _stream(stream)))


def sigmadelta(frame, bkg, var, label, stream=None):
    check(load().nt2g_sigmadelta_u8(_ptr(frame), _ptr(bkg), _ptr(var), _ptr(label), frame.numel(),
                                    _stream(stream)))


def sigmadelta_frames(frames, bkg, var, labels, stream=None):
    nf = frames.shape[0]
    check(load().nt2g_sigmadelta_frames_u8(_ptr(frames), _ptr(bkg), _ptr(var), _ptr(labels), bkg.numel(), nf,
                                           _stream(stream)))


def map_f32(fn, x, y, precision=PREC_FAST, stream=None):
    check(load().nt2g_map_f32(MAP_FN[fn], _ptr(x), _ptr(y), x.numel(), precision, _stream(stream)))


FOLD = {"sum": 0, "prod": 1, "max": 2, "min": 3, "mean": 4, "asum1": 5, "asum2": 6, "norm2": 7, "var": 8, "stdev": 9,
        "var1": 10, "stdev1": 11, "nbtrue": 12, "all": 13, "any": 14, "none": 15, "nansum": 16, "nanmean": 17, "meanad": 18}


def fold(x, lo, inner, hi, op, precision=PREC_FAST, index=False, stream=None):
    """Reduce x (viewed as [lo, inner, hi], column-major) over inner:
    returns out[lo*hi] (and the int64 first-equal index for max/min)."""
    import torch
    nb = ctypes.c_size_t()
    check(load().nt2g_fold_workspace_size(lo, inner, hi, ctypes.byref(nb)))
    dev = x.device
    ws = torch.empty(max(nb.value, 16), dtype=torch.uint8, device=dev)
    out = torch.empty(lo * hi, dtype=torch.float32, device=dev)
    idx = torch.empty(lo * hi, dtype=torch.int64, device=dev) if index else None
    check(load().nt2g_fold_f32(_ptr(x), lo, inner, hi, FOLD[op], precision, _ptr(ws), ws.numel(), _ptr(out),
                               _ptr(idx), _stream(stream)))
    return (out, idx) if index else out


MEDIAN = {"median": 0, "medianad": 1}


def trapz(x, lo, inner, hi, precision=PREC_FAST, stream=None):
    """NT2's trapz (unit spacing) of x viewed as [lo, inner, hi] along inner: out[lo*hi]."""
    import torch
    nb = ctypes.c_size_t()
    check(load().nt2g_trapz_workspace_size(lo, inner, hi, ctypes.byref(nb)))
    ws = torch.empty(max(nb.value, 16), dtype=torch.uint8, device=x.device)
    out = torch.empty(lo * hi, dtype=torch.float32, device=x.device)
    check(load().nt2g_trapz_f32(_ptr(x), lo, inner, hi, precision, _ptr(ws), ws.numel(), _ptr(out), _stream(stream)))
    return out


def median(x, lo, inner, hi, op="median", out=None, stream=None):
    """NT2's median (or medianad) of x viewed as [lo, inner, hi] along inner:
    returns out[lo*hi]."""
    import torch
    nb = ctypes.c_size_t()
    check(load().nt2g_median_workspace_size(lo, inner, hi, ctypes.byref(nb)))
    ws = torch.empty(max(nb.value, 16), dtype=torch.uint8, device=x.device)
    out = torch.empty(lo * hi, dtype=torch.float32, device=x.device) if out is None else out
    check(load().nt2g_median_f32(_ptr(x), lo, inner, hi, MEDIAN[op], _ptr(ws), ws.numel(), _ptr(out),
                                 _stream(stream)))
    return out


SCAN = {"sum": 0, "prod": 1, "max": 2, "min": 3}


def scan(x, lo, inner, hi, op, precision=PREC_FAST, out=None, stream=None):
    """Cumulative op of x viewed as [lo, inner, hi] along inner (cumsum, cumprod,
    cummax, cummin); out may be x."""
    import torch
    nb = ctypes.c_size_t()
    check(load().nt2g_scan_workspace_size(lo, inner, hi, ctypes.byref(nb)))
    ws = torch.empty(max(nb.value, 16), dtype=torch.uint8, device=x.device)
    out = torch.empty_like(x) if out is None else out
    check(load().nt2g_scan_f32(_ptr(x), lo, inner, hi, SCAN[op], precision, _ptr(ws), ws.numel(), _ptr(out),
                               _stream(stream)))
    return out


class Reducer:
    """sum / dot with a workspace allocated once (through torch)."""

    def __init__(self, device="cuda"):
        import torch
        nb = ctypes.c_size_t()
        check(load().nt2g_reduce_workspace_size(0, ctypes.byref(nb)))
        self.ws = torch.empty(nb.value, dtype=torch.uint8, device=device)
        self.out64 = torch.zeros(1, dtype=torch.float64, device=device)
        self.out32 = torch.zeros(1, dtype=torch.float32, device=device)

    def __call__(self, x, y=None, stream=None):
        check(load().nt2g_reduce_f32(_ptr(x), _ptr(y), x.numel(), _ptr(self.ws), self.ws.numel(),
                                     _ptr(self.out64), _ptr(self.out32), _stream(stream)))
        return self.out64, self.out32
