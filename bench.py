#!/usr/bin/env python3
"""Throughput of the fused-expression evaluator on GB300.

python bench.py [--gpus N] [--steps K] [--warmup W] [--config NAME] [--impl ours|reference]

A step is one pass of the hot path over one batch of synthetic input resident
in HBM.  Workloads (--config):
  bs        (default) fused Black-Scholes call+put, N=1,048,576 options per
            step, S~U[5,30] K~U[1,100] T~U[0.25,10], r=0.02, sigma=0.30.  A
            20 MB batch fits in L2, so steps rotate over 32 input/output sets
            (640 MB) and every step reads HBM.
  reduce    dot(x,y) over 2^28 float32, x,y ~ N(0,1) (2 GiB per step)
  sum       sum(x) over 2^28 float32
  batched   4096 tables, sizes log-uniform in [1024, 4194304], one of BS /
            saxpy / expr3 each; one persistent launch per step
  pertable  the same batch, one plain launch per table per step
  batched_programs  the same batch with every table a user program (its
            expression written out), linked into one compiled batch kernel
  adjoint   fused BS forward + reverse (VJP), N=2^26 options
  adjoint_fwd  the forward alone on the same options (the 2.2x reference)
  bs_demo   NT2's demo Black-Scholes (call only, fastnormcdf), 2^20 options per step
  adjoint_program / adjoint_demo   reverse mode of a user program (nt2g_program_vjp)
            on 2^26 options: textbook BS (sigma table, r scalar) / NT2's demo form
  sigmadelta   1920x1080 uint8 frames, one fused step per frame
  sigmadelta_fused  63 frame steps in one kernel
  rgb2yuv   1920x1080x3 float planes
  bs_generic / bs_interp   the bs batch through the expression API's compiled
            kernel / interpreter (fused binding skipped)
  fold_col / fold_row / gmax   sum(A, 1), sum(A, 2), globalmax of a 16384^2 table
  cumsum_col / cumsum_all / cummax_row   cumulative functions on that table
  median_col / median_row / gmedian   median(A, 1), median(A, 2), globalmedian of that table
  fn_trig / fn_pow / fn_gen   sin(x)*cos(y), pow(x, y), sinpi(linspace(0,2,n))*x
  fn_special                  erf(y) + gammaln(x)
            over 2^26 elements through the compiled kernel
  fold_expr / fold_expr_col   sum(exp(x)*y) over 2^28 elements, sum(abs(x - y), 1)
            of two 16384^2 tables: folds of an expression in one pass
Each prints one JSON line (rank 0).  --impl reference times NT2's CPU path
(the oracle's restatement of it: NT2 itself needs Boost, absent here) on the
host cores for the same workload.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "elements/s and % of HBM peak, fused exprs: plain vs batched/adjoint at ≤4 ulp"
UNIT = "elements/s"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel_key):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        d = json.load(open(p))
        v = d.get(kernel_key)
        if isinstance(v, dict):
            return v.get("bytes_per_launch")
        return v
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.proc, self.lines = index, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 6:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[2:6]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


# -------------------------------------------------------- multi-rank logic
def max_over_ranks(ms, world, dist=None, device="cpu"):
    """Slowest rank's time: every rank must have finished its batch."""
    if world == 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(units_per_rank, steps, world, ms):
    """Elements per second over all ranks (replicas: each rank its own batch)."""
    return world * units_per_rank * steps / (ms / 1e3)


# ----------------------------------------------------------------- workloads
class Workload:
    name = ""
    units = 0          # elements per step
    bytes = 0          # algorithmic HBM bytes per step
    launches = 1       # our kernels per step
    kernel = ""        # dominant kernel (for the roofline)
    flush = "inputs larger than L2"
    independent = False  # consecutive steps touch disjoint buffers (may overlap on two streams)

    def step(self, i):
        raise NotImplementedError


class BlackScholes(Workload):
    N = 1 << 20
    SETS = 32
    independent = True

    def __init__(self, torch, lib, dev, precision, n=None):
        self.torch, self.lib, self.prec = torch, lib, precision
        if n:  # options per launch other than the standard 2^20; enough sets to exceed 640 MiB
            self.N = int(n)
            self.SETS = max(2, -(-(640 << 20) // (20 * self.N)))
        self.name = f"blackscholes_plain N={self.N} call+put, {self.SETS} rotating sets"
        self.units, self.bytes, self.kernel = self.N, 20 * self.N, "k_bs"
        self.flush = f"rotating {self.SETS} input/output sets ({self.SETS * 20 * self.N >> 20} MiB > L2)"
        g = torch.Generator(device=dev).manual_seed(1000)
        self.S = torch.rand(self.SETS, self.N, device=dev, generator=g) * 25 + 5
        self.K = torch.rand(self.SETS, self.N, device=dev, generator=g) * 99 + 1
        self.T = torch.rand(self.SETS, self.N, device=dev, generator=g) * 9.75 + 0.25
        self.C = torch.empty_like(self.S)
        self.P = torch.empty_like(self.S)

    def step(self, i):
        k = i % self.SETS
        self.lib.blackscholes(self.S[k], self.K[k], self.T[k], self.C[k], self.P[k], 0.02, sigma_s=0.30,
                              precision=self.prec)

    # End to end through the C ABI on HOST tables: each step prices one of
    # HOST_SETS rotating sets of pinned host tables (320 MiB > L2) in place --
    # the kernel reads S, K, T from host memory and writes call, put back over
    # the host link (NVLink-C2C on Grace-Blackwell) with no staging copy.
    # Steps rotate over four streams: a host-memory launch is latency-bound at
    # its ramp and tail, and concurrent launches keep the link busy.
    LANES = 4
    HOST_SETS = 16

    def e2e_setup(self):
        t = self.torch
        self.host = []
        for k in range(self.HOST_SETS):
            j = k % self.SETS
            ins = [self.S[j].cpu().pin_memory(), self.K[j].cpu().pin_memory(), self.T[j].cpu().pin_memory()]
            outs = [t.empty(self.N, pin_memory=True), t.empty(self.N, pin_memory=True)]
            self.host.append((ins, outs))
        self.lanes = [t.cuda.Stream() for _ in range(self.LANES)]
        return 12 * self.N, 8 * self.N

    def e2e_call(self, ins, outs, stream):
        self.lib.blackscholes(ins[0], ins[1], ins[2], outs[0], outs[1], 0.02, sigma_s=0.30, precision=self.prec,
                              stream=stream)

    def e2e_step(self, i):
        ins, outs = self.host[i % self.HOST_SETS]
        st = self.lanes[i % self.LANES]
        with self.torch.cuda.stream(st):
            self.e2e_call(ins, outs, st)

    def e2e_streams(self):
        return self.lanes

    @staticmethod
    def cpu(oracle, nthreads, sample_n, inputs=None):
        if inputs is None:
            rng = np.random.default_rng(1000)
            S = rng.uniform(5, 30, sample_n).astype(np.float32)
            K = rng.uniform(1, 100, sample_n).astype(np.float32)
            T = rng.uniform(0.25, 10, sample_n).astype(np.float32)
        else:
            S, K, T = inputs
        return lambda: oracle.blackscholes(S, K, T, 0.02, 0.30, nthreads=nthreads)

    def sample(self):
        """Inputs and timed outputs of rotating set 0 (host copies)."""
        ins = tuple(a[0].cpu().numpy() for a in (self.S, self.K, self.T))
        return ins, (self.C[0].cpu().numpy(), self.P[0].cpu().numpy())

    def accuracy(self, nt2_out=None):
        (S, K, T), (c, p) = self.sample()
        return bs_accuracy(S, K, T, c, p, 0.02, 0.30, self.prec, nt2_out)


# ----------------------------------------------------------------- accuracy
def bs_fp64(S, K, T, r, sigma):
    """Black-Scholes call, put and the four cancelling terms in FP64 (the same
    formula; sigma and r as the float32 values the kernel receives)."""
    try:
        from scipy.special import erfc
    except ImportError:  # pragma: no cover - scipy is present on both machines
        import math
        erfc = np.vectorize(math.erfc)
    s, k, t = (np.asarray(a, np.float64) for a in (S, K, T))
    v, rr = float(np.float32(sigma)), float(np.float32(r))
    sq = np.sqrt(t)
    d1 = (np.log(s / k) + (rr + 0.5 * v * v) * t) / (v * sq)
    d2 = d1 - v * sq
    e = k * np.exp(-rr * t)
    N = lambda x: 0.5 * erfc(-x / np.sqrt(2.0))  # noqa: E731
    a, b, c, d = s * N(d1), e * N(d2), e * N(-d2), s * N(-d1)
    return a - b, c - d, (a, b, c, d)


def bs_accuracy(S, K, T, call, put, r, sigma, precision, nt2_out=None):
    """Error of the timed outputs against FP64 in conditioned ulps: |error| in
    ulps of the larger of the two cancelling terms (call = S N(d1) - K e^-rT
    N(d2)), terms floored at 2^-102 where N(d) is subnormal in FP32.  With
    nt2_out (NT2's CPU evaluation of the same options), whether the outputs
    are bit-identical to it."""
    c64, p64, (a, b, c, d) = bs_fp64(S, K, T, r, sigma)
    floor = 2.0 ** -102
    out = {"vs": "FP64 evaluation of the same formula (numpy/scipy)", "metric": "conditioned ulp",
           "sample": f"rotating set 0 ({np.asarray(S).size} options) after the timed steps"}
    for name, got, ref, t1, t2 in (("call", call, c64, a, b), ("put", put, p64, c, d)):
        scale = np.maximum(np.maximum(np.abs(t1), np.abs(t2)), floor).astype(np.float32)
        e = np.abs(np.asarray(got, np.float64) - ref) / np.spacing(scale).astype(np.float64)
        out[name] = {"max": float(e.max()), "mean": float(e.mean()), "p99.9": float(np.quantile(e, 0.999))}
    if nt2_out is not None:
        same = all(np.array_equal(np.asarray(g, np.float32).view(np.uint32), np.asarray(o, np.float32).view(np.uint32))
                   for g, o in zip((call, put), nt2_out))
        out["nt2_bit_exact"] = bool(same)
    out["stated"] = BS_TOLERANCE["nt2" if precision == 1 else "fast"]
    return out


BS_TOLERANCE = {
    "nt2": "bit-identical to NT2's CPU evaluation (the CPU baseline leg evaluates the same options)",
    "fast": "every functor within 4 ulp of FP64; the composite call/put within 14 conditioned ulp max, "
            "6 at p99.9, 1.1 mean (error over the ulp of the larger cancelling term); NT2's own float "
            "evaluation of the same options: about 300 max, 90 p99.9, 3.4 mean",
}


class BlackScholesGeneric(BlackScholes):
    """The same batch through the expression front end with the fused-kernel
    binding skipped: the program's run-time compiled kernel (mode 1) or the
    generic interpreter (mode 2)."""

    def __init__(self, torch, lib, dev, precision, mode=1, n=None):
        super().__init__(torch, lib, dev, precision, n)
        from nt2_gb300 import expr as E
        self.E, self.mode = E, mode
        what = "run-time compiled kernel" if mode == 1 else "generic interpreter"
        self.name = f"blackscholes_plain N={self.N} call+put through the {what}, {self.SETS} sets"
        self.kernel = "nt2g_jit_kernel" if mode == 1 else "k_interp"

    def step(self, i):
        E, k = self.E, i % self.SETS
        S, K, T = E.Table(self.S[k]), E.Table(self.K[k]), E.Table(self.T[k])
        sig, r = 0.30, 0.02
        sq = E.sqrt(T)
        d1 = (E.log(S / K) + E.fma(E.sqr(sig), 0.5, r) * T) / (sig * sq)
        d2 = E.fnms(sig, sq, d1)
        e = K * E.exp(-r * T)
        prog = E.assign([self.C[k], self.P[k]], [E.fnms(e, E.normcdf(d2), S * E.normcdf(d1)),
                                                E.fnms(S, E.normcdf(-d1), e * E.normcdf(-d2))],
                        precision=self.prec, force_generic=self.mode)
        if self.mode == 1 and i == 0:
            prog.jit_prepare(self.prec)  # fail loudly rather than time the interpreter

    def e2e_call(self, ins, outs, stream):
        E = self.E
        S, K, T = E.Table(ins[0]), E.Table(ins[1]), E.Table(ins[2])
        sig, r = 0.30, 0.02
        sq = E.sqrt(T)
        d1 = (E.log(S / K) + E.fma(E.sqr(sig), 0.5, r) * T) / (sig * sq)
        d2 = E.fnms(sig, sq, d1)
        e = K * E.exp(-r * T)
        E.assign([outs[0], outs[1]], [E.fnms(e, E.normcdf(d2), S * E.normcdf(d1)),
                                      E.fnms(S, E.normcdf(-d1), e * E.normcdf(-d2))],
                 precision=self.prec, force_generic=self.mode, stream=stream)


class BlackScholesDemo(BlackScholes):
    """NT2's demo Black-Scholes as its source writes it
    (demo/blackscholes/nt2/blackandscholes_nt2.cpp:55-59): call only,
    fastnormcdf, d1 = log(S/X) + fma(v^2, 1/2, r) T / (v sqrt(T)); S, X, T
    tables, r = 0.02 and v = 0.30 scalars: 16 B/option (three tables read, one
    written), the same rotating 2^20-option sets."""

    def __init__(self, torch, lib, dev, precision, n=None):
        super().__init__(torch, lib, dev, precision, n)
        self.name = f"blackscholes NT2 demo form N={self.N} call only (fastnormcdf), {self.SETS} rotating sets"
        self.bytes, self.kernel = 16 * self.N, "k_bs_demo"

    def step(self, i):
        k = i % self.SETS
        self.lib.blackscholes_demo(self.S[k], self.K[k], self.T[k], self.C[k], r=0.02, v=0.30, precision=self.prec)

    def e2e_setup(self):
        h2d, _ = super().e2e_setup()
        return h2d, 4 * self.N

    def e2e_call(self, ins, outs, stream):
        self.lib.blackscholes_demo(ins[0], ins[1], ins[2], outs[0], r=0.02, v=0.30, precision=self.prec,
                                   stream=stream)

    cpu = None
    accuracy = None


class Reduce(Workload):
    N = 1 << 28

    def __init__(self, torch, lib, dev, dot=True):
        self.torch, self.lib, self.dot = torch, lib, dot
        self.name = f"{'dot' if dot else 'sum'} n=2^28 float32 N(0,1), compensated FP32 + FP64 block combine"
        self.units, self.bytes, self.kernel = self.N, (8 if dot else 4) * self.N, "k_reduce"
        g = torch.Generator(device=dev).manual_seed(1001)
        self.x = torch.randn(self.N, device=dev, generator=g)
        self.y = torch.randn(self.N, device=dev, generator=g) if dot else None
        self.red = lib.Reducer(dev)

    def step(self, i):
        self.red(self.x, self.y)


def _bs_program_exprs(E, S, K, T, sig, r):
    """Black-Scholes call/put as NT2 writes the expression (the textbook form)."""
    sq = E.sqrt(T)
    d1 = (E.log(S / K) + E.fma(E.sqr(sig), 0.5, r) * T) / (sig * sq)
    d2 = E.fnms(sig, sq, d1)
    e = K * E.exp(-r * T)
    return [E.fnms(e, E.normcdf(d2), S * E.normcdf(d1)), E.fnms(S, E.normcdf(-d1), e * E.normcdf(-d2))]


class Batched(Workload):
    def __init__(self, torch, lib, dev, per_table=False, precision=0, tune=None, programs=False):
        from tests.helpers import batched_sizes
        self.torch, self.lib, self.per_table = torch, lib, per_table
        sizes, exprs = batched_sizes()
        self.sizes, self.exprs = sizes, exprs
        g = torch.Generator(device=dev).manual_seed(1003)
        self.tabs, self.keep = [], []
        items = (lib.BatchItem * len(sizes))()
        total_bytes = 0
        for i, (n, ex) in enumerate(zip(sizes, exprs)):
            n = int(n)
            if ex == lib.BATCH_BLACKSCHOLES:
                ins = [torch.rand(n, device=dev, generator=g) * 25 + 5, torch.rand(n, device=dev, generator=g) * 99 + 1,
                       torch.rand(n, device=dev, generator=g) * 9.75 + 0.25]
                outs = [torch.empty(n, device=dev), torch.empty(n, device=dev)]
                s = (0.30, 0.02)
                total_bytes += 20 * n
            elif ex == lib.BATCH_SAXPY:
                ins = [torch.randn(n, device=dev, generator=g)]
                outs = [torch.randn(n, device=dev, generator=g)]
                s = (float(np.float32(np.random.default_rng(i).uniform(-2, 2))), 0.0)
                total_bytes += 12 * n
            else:
                ins = [torch.randn(n, device=dev, generator=g) for _ in range(3)]
                outs = [torch.empty(n, device=dev)]
                s = (0.0, 0.0)
                total_bytes += 16 * n
            self.tabs.append((ins, outs))
            if programs:  # the same table as a user program (its expression written out)
                from nt2_gb300 import expr as E
                T = [E.Table(t) for t in ins]
                if ex == lib.BATCH_BLACKSCHOLES:
                    ex_outs = _bs_program_exprs(E, T[0], T[1], T[2], E.Scalar(s[0]), E.Scalar(s[1]))
                elif ex == lib.BATCH_SAXPY:
                    ex_outs = [E.Scalar(s[0]) * T[0] + E.Table(outs[0])]
                else:
                    ex_outs = [E.exp(-E.sqr(T[0])) * E.sqrt(E.abs_(T[1])) + E.log1p(E.abs_(T[2]))]
                it, prog, args = E.batch_item(outs, ex_outs)
                self.keep.append((prog, args))
                items[i] = it
                continue
            items[i].expr, items[i].n = int(ex), n
            for j, t in enumerate(ins):
                items[i].inp[j] = t.data_ptr()
            for j, t in enumerate(outs):
                items[i].out[j] = t.data_ptr()
            items[i].s[0], items[i].s[1] = s
        if tune:
            tn, how = tune, "given"
        else:  # the project's autotuner, cached per GPU and batch shape
            from nt2_gb300 import autotune
            best, _, cached = autotune.tuned(items, precision)
            tn, how = (best.block_threads, best.blocks_per_sm, best.tile_vectors, best.vector_width), \
                ("autotuned (cache)" if cached else "autotuned")
        t = lib.BatchTune(tn[0], tn[1], tn[2], precision, tn[3] if len(tn) > 3 else 1)
        self.h = ctypes.c_void_p()
        lib.check(lib.load().nt2g_batch_create(items, len(sizes), ctypes.byref(t), ctypes.byref(self.h)))
        self.units = int(np.sum(sizes))
        self.bytes = total_bytes
        self.launches = len(sizes) if per_table else 1
        self.kernel = "k_single" if per_table else ("batch_" if programs else "k_batch")
        self.name = (f"batched 4096 tables log-uniform [1024, 4194304] ({self.units} elements)"
                     f"{', every table a user program' if programs else ''}, "
                     f"{'one plain launch per table' if per_table else 'one persistent launch'}, "
                     f"tune threads,blocks/SM,vectors/tile,vectors/step={tn} ({how})")

    def step(self, i):
        fn = self.lib.load().nt2g_batch_run_per_table if self.per_table else self.lib.load().nt2g_batch_run
        self.lib.check(fn(self.h, self.lib._stream()))


class Adjoint(Workload):
    N = 1 << 26

    def __init__(self, torch, lib, dev, forward_only=False):
        self.torch, self.lib, self.fwd = torch, lib, forward_only
        g = torch.Generator(device=dev).manual_seed(1004)
        n = self.N
        self.S = torch.rand(n, device=dev, generator=g) * 25 + 5
        self.K = torch.rand(n, device=dev, generator=g) * 99 + 1
        self.T = torch.rand(n, device=dev, generator=g) * 9.75 + 0.25
        self.sig = torch.rand(n, device=dev, generator=g) * 0.75 + 0.05
        self.gc = torch.rand(n, device=dev, generator=g) * 2 - 1
        self.gp = torch.rand(n, device=dev, generator=g) * 2 - 1
        self.outs = [torch.empty(n, device=dev) for _ in range(7)]
        self.units = n
        self.bytes = (24 if forward_only else 52) * n
        self.kernel = "k_bs" if forward_only else "k_bs_vjp"
        self.name = (f"blackscholes {'forward' if forward_only else 'forward+VJP'} N=2^26, sigma table")

    def step(self, i):
        if self.fwd:
            self.lib.blackscholes(self.S, self.K, self.T, self.outs[0], self.outs[1], 0.02, sigma=self.sig)
        else:
            self.lib.blackscholes_vjp(self.S, self.K, self.T, self.sig, 0.02, self.gc, self.gp, self.outs)


class ProgramAdjoint(Workload):
    """Reverse mode of a user program (nt2g_program_vjp) over 2^26 options:
    the textbook Black-Scholes call and put (sigma a table, r a scalar, both
    cotangents; gradients of S, K, T, sigma and the summed dr), or the NT2
    demo form (all five inputs tables, one cotangent).  Forward values are
    recomputed in registers: nothing but the inputs, the cotangents and the
    gradients moves."""
    N = 1 << 26

    def __init__(self, torch, lib, dev, form="textbook", precision=0):
        import ctypes as C
        from nt2_gb300 import expr as E
        self.torch, self.lib = torch, lib
        g = torch.Generator(device=dev).manual_seed(1004)
        n = self.N
        rnd = lambda lo, hi: torch.rand(n, device=dev, generator=g) * (hi - lo) + lo  # noqa: E731
        if form == "textbook":
            S, K, T, sig = rnd(5, 30), rnd(1, 100), rnd(0.25, 10), rnd(0.05, 0.8)
            cts = [rnd(-1, 1), rnd(-1, 1)]
            outs = [torch.empty(n, device=dev), torch.empty(n, device=dev)]
            St, Kt, Tt, st = (E.Table(x) for x in (S, K, T, sig))
            rs = E.Scalar(0.02)
            exprs = _bs_program_exprs(E, St, Kt, Tt, st, rs)
            wrt = [S, K, T, sig]
            self.bytes = (6 * 4 + 4 * 4) * n
            what = "textbook call+put, sigma table, r scalar: dS dK dT dsigma (tables) + dr (summed)"
        else:
            S, X, T, r, v = rnd(5, 30), rnd(1, 100), rnd(0.25, 10), rnd(0.01, 0.05), rnd(0.1, 0.6)
            cts = [rnd(-1, 1)]
            outs = [torch.empty(n, device=dev)]
            da = E.sqrt(E.Table(T))
            Sa, Xa, Ta, ra, va = (E.Table(x) for x in (S, X, T, r, v))
            d1 = E.log(Sa / Xa) + (E.fma(E.sqr(va), 0.5, ra) * Ta) / (va * da)
            d2 = E.fnms(va, da, d1)
            exprs = [E.fnms(Xa * E.exp(-ra * Ta), E.fastnormcdf(d2), Sa * E.fastnormcdf(d1))]
            wrt = [S, X, T, r, v]
            self.bytes = (6 * 4 + 5 * 4) * n
            what = "NT2 demo form, five input tables: all five gradients"
        self.keep = (S, T, cts, outs, wrt, exprs)
        prog, slots = E.compile_program(outs, exprs)
        self.prog = prog
        self.args, _ = E._args_of(slots)
        ns = len(slots)
        self.ns = ns
        self.ct, self.tg = (C.c_void_p * ns)(), (C.c_void_p * ns)()
        for o, c in zip(outs, cts):
            self.ct[E._slot_of(slots, o)] = c.data_ptr()
        self.grads = []
        for x in wrt:
            gx = torch.empty_like(x)
            self.tg[E._slot_of(slots, x)] = gx.data_ptr()
            self.grads.append(gx)
        self.sg = torch.zeros(ns, dtype=torch.float64, device=dev)
        nb = C.c_size_t()
        lib.check(lib.load().nt2g_program_vjp_workspace_size(prog.handle, n, C.byref(nb)))
        self.ws = torch.empty(max(nb.value, 16), dtype=torch.uint8, device=dev)
        self.prec = precision
        self.units = n
        self.launches = 2 if form == "textbook" else 1  # + the scalar gradients' fixed-order sum
        self.kernel = "nt2g_vjp_kernel"
        self.name = f"program VJP N=2^26, {what}"

    def step(self, i):
        L = self.lib
        L.check(L.load().nt2g_program_vjp(self.prog.handle, self.args, self.ns, self.N, self.ct, self.tg,
                                          L._ptr(self.sg), self.prec, L._ptr(self.ws), self.ws.numel(), L._stream()))


class SigmaDelta(Workload):
    def __init__(self, torch, lib, dev):
        self.torch, self.lib = torch, lib
        h, w, f = 1080, 1920, 64
        g = torch.Generator(device=dev).manual_seed(1002)
        self.frames = torch.randint(0, 256, (f, h * w), dtype=torch.uint8, device=dev, generator=g)
        self.bkg = self.frames[0].clone()
        self.var = torch.ones_like(self.bkg)
        self.lab = torch.empty_like(self.bkg)
        self.units, self.bytes, self.kernel = h * w, 6 * h * w, "k_sigmadelta"
        self.name = "sigmadelta 1920x1080 uint8, one frame per step over 64 frames"
        self.flush = "64 frames (132 MB) rotated"

    def step(self, i):
        self.lib.sigmadelta(self.frames[1 + i % 63], self.bkg, self.var, self.lab)


class SigmaDeltaFused(Workload):
    """All 63 frame steps of the 64-frame sequence in one launch: bkg/var stay
    in registers, each frame is read and each label written once."""

    def __init__(self, torch, lib, dev):
        self.torch, self.lib = torch, lib
        h, w, f = 1080, 1920, 64
        g = torch.Generator(device=dev).manual_seed(1002)
        self.frames = torch.randint(0, 256, (f, h * w), dtype=torch.uint8, device=dev, generator=g)
        self.bkg = self.frames[0].clone()
        self.var = torch.ones_like(self.bkg)
        self.labels = torch.empty((f - 1, h * w), dtype=torch.uint8, device=dev)
        nf = f - 1
        self.units = h * w * nf
        self.bytes = h * w * (2 * nf + 4)
        self.kernel = "k_sigmadelta_frames"
        self.name = "sigmadelta 1920x1080 uint8, 63 frame steps fused in one launch per step"

    def step(self, i):
        self.lib.sigmadelta_frames(self.frames[1:], self.bkg, self.var, self.labels)


class Fold(Workload):
    """Reduction along one dimension of a 16384 x 16384 float table (1 GiB):
    dim 1 = per-column (contiguous) sums, dim 2 = per-row (strided) sums; or a
    global max over the same 2^28 elements."""

    def __init__(self, torch, lib, dev, kind, precision, side=16384):
        import ctypes
        self.torch, self.lib, self.prec = torch, lib, precision
        m = n = side
        g = torch.Generator(device=dev).manual_seed(1001)
        self.x = torch.randn(m * n, device=dev, generator=g)
        self.shape = {"col": (1, m, n), "row": (m, n, 1), "max": (1, m * n, 1)}[kind]
        self.op = lib.FOLD["max" if kind == "max" else "sum"]
        lo, inner, hi = self.shape
        nb = ctypes.c_size_t()
        lib.check(lib.load().nt2g_fold_workspace_size(lo, inner, hi, ctypes.byref(nb)))
        self.ws = torch.empty(max(nb.value, 16), dtype=torch.uint8, device=dev)
        self.out = torch.empty(lo * hi, device=dev)
        self.units = m * n
        self.bytes = 4 * m * n + 4 * lo * hi
        self.kernel = {"col": "k_fold_inner", "row": "k_fold_outer", "max": "k_fold_inner"}[kind]
        self.launches = 1 if kind == "col" else 2  # strided and global folds add the in-order combine
        what = {"col": f"sum(A, 1): {n} column sums", "row": f"sum(A, 2): {m} row sums",
                "max": f"globalmax over {m * n}"}[kind]
        self.name = f"fold {what} of a {m}x{n} float32 table"
        self.flush = f"{4 * m * n >> 20} MiB input" + (" > L2" if 4 * m * n > 129 << 20 else " (below L2)")

    def step(self, i):
        lo, inner, hi = self.shape
        L = self.lib
        L.check(L.load().nt2g_fold_f32(L._ptr(self.x), lo, inner, hi, self.op, self.prec, L._ptr(self.ws),
                                       self.ws.numel(), L._ptr(self.out), None, L._stream()))


class Median(Workload):
    """median(A, 1) (column slices, each held in one block's shared memory),
    median(A, 2) (strided row slices) or globalmedian (all elements: four
    histogram passes and a successor pass over global memory) of a
    16384 x 16384 float table.  Algorithmic bytes: the table read once plus the
    medians written."""

    def __init__(self, torch, lib, dev, kind, side=16384):
        import ctypes
        self.torch, self.lib = torch, lib
        m = n = side
        g = torch.Generator(device=dev).manual_seed(1003)
        self.x = torch.randn(m * n, device=dev, generator=g)
        self.shape = {"col": (1, m, n), "row": (m, n, 1), "all": (1, m * n, 1)}[kind]
        lo, inner, hi = self.shape
        nb = ctypes.c_size_t()
        lib.check(lib.load().nt2g_median_workspace_size(lo, inner, hi, ctypes.byref(nb)))
        self.ws = torch.empty(max(nb.value, 16), dtype=torch.uint8, device=dev)
        self.out = torch.empty(lo * hi, device=dev)
        self.units = m * n
        self.bytes = 4 * m * n + 4 * lo * hi
        glob = nb.value > 0
        self.kernel = "k_median_hist" if glob else "k_median_smem"
        self.launches = 11 if glob else 1  # init, 4 x (histogram, pick), successor, output
        what = {"col": f"median(A, 1): {n} column medians", "row": f"median(A, 2): {m} row medians",
                "all": f"globalmedian over {m * n}"}[kind]
        self.name = f"{what} of a {m}x{n} float32 table"
        self.flush = f"{4 * m * n >> 20} MiB input" + (" > L2" if 4 * m * n > 129 << 20 else " (below L2)")

    def step(self, i):
        lo, inner, hi = self.shape
        L = self.lib
        L.check(L.load().nt2g_median_f32(L._ptr(self.x), lo, inner, hi, 0, L._ptr(self.ws), self.ws.numel(),
                                         L._ptr(self.out), L._stream()))


class Scan(Workload):
    """Cumulative op along one dimension of a 16384 x 16384 float table
    (1 GiB in, 1 GiB out: 8 B/element algorithmic): cumsum per column, cumsum
    of the whole table as one segment, or cummax per row (strided)."""

    def __init__(self, torch, lib, dev, kind, precision, side=16384):
        import ctypes
        self.torch, self.lib, self.prec = torch, lib, precision
        m = n = side
        g = torch.Generator(device=dev).manual_seed(1001)
        self.x = torch.randn(m * n, device=dev, generator=g)
        self.y = torch.empty_like(self.x)
        self.shape = {"col": (1, m, n), "all": (1, m * n, 1), "rowmax": (m, n, 1)}[kind]
        self.op = lib.SCAN["max" if kind == "rowmax" else "sum"]
        lo, inner, hi = self.shape
        nb = ctypes.c_size_t()
        lib.check(lib.load().nt2g_scan_workspace_size(lo, inner, hi, ctypes.byref(nb)))
        self.ws = torch.empty(max(nb.value, 16), dtype=torch.uint8, device=dev)
        self.units, self.bytes = m * n, 8 * m * n
        self.kernel = "k_scan_outer" if kind == "rowmax" else "k_scan_inner"
        self.launches = 1 if nb.value == 0 else 3
        what = {"col": f"cumsum(A, 1): {n} columns", "all": f"cumsum over all {m * n} elements (one segment)",
                "rowmax": f"cummax(A, 2): {m} rows, strided"}[kind]
        self.name = f"scan {what} of a {m}x{n} float32 table"
        self.flush = f"{4 * m * n >> 20} MiB input" + (" > L2" if 4 * m * n > 129 << 20 else " (below L2)")

    def step(self, i):
        lo, inner, hi = self.shape
        L = self.lib
        L.check(L.load().nt2g_scan_f32(L._ptr(self.x), lo, inner, hi, self.op, self.prec, L._ptr(self.ws),
                                       self.ws.numel(), L._ptr(self.y), L._stream()))


class Functors(Workload):
    """A generic expression of the newer functors through the run-time compiled
    kernel (the path any user expression takes), fast policy, over 2^26-element
    tables: sin(x) * cos(y), pow(x, y), sinpi(linspace(0, 2, n)) * x (a
    generative leaf: no input bytes for it), or erf(y) + gammaln(x)."""

    def __init__(self, torch, lib, dev, kind, precision, n=None):
        from nt2_gb300 import expr as E
        self.torch, self.lib, self.prec = torch, lib, precision
        n = n or 1 << 26
        g = torch.Generator(device=dev).manual_seed(1003)
        self.x = torch.rand(n, device=dev, generator=g) * 4 + 0.25
        self.y = torch.rand(n, device=dev, generator=g) * 4 - 2
        self.out = torch.empty_like(self.x)
        X, Y = E.Table(self.x), E.Table(self.y)
        e = {"trig": E.sin(X) * E.cos(Y), "pow": E.pow(X, Y), "gen": E.sinpi(E.linspace(0, 2, n)) * X,
             "special": E.erf(Y) + E.gammaln(X)}[kind]
        prog, slots = E.compile_program([self.out], [e])
        prog.jit_prepare(precision)
        self.prog = prog
        self.args = (lib.Arg * len(slots))(*[lib.Arg(t.data_ptr(), 0.0, lib.F32, 0) for t in slots])
        self.nslots, self.n = len(slots), n
        reads = {"trig": 8, "pow": 8, "gen": 4, "special": 8}[kind]
        self.units, self.bytes, self.kernel = n, (reads + 4) * n, "nt2g_jit_kernel"
        self.name = {"trig": "sin(x) * cos(y)", "pow": "pow(x, y)", "gen": "sinpi(linspace(0, 2, n)) * x",
                     "special": "erf(y) + gammaln(x)"}[kind] + \
            f" over {n} float32 elements, run-time compiled kernel"
        self.flush = "inputs larger than L2"

    def step(self, i):
        L = self.lib
        L.check(L.load().nt2g_eval(self.prog.handle, self.args, self.nslots, 0, self.n, self.prec, 1, L._stream()))


class FoldExpr(Workload):
    """A fold of an expression in one pass (nt2g_eval_fold): the expression is
    evaluated inside the fold kernels, so the algorithmic bytes are the input
    tables' only (8 B/element, no temporary).  kind "sum": sum(exp(x)*y) over
    2^28 elements (FP64 result); kind "col": sum(abs(x - y), 1) over a
    16384 x 16384 table (16384 column sums)."""

    def __init__(self, torch, lib, dev, kind, precision, n=None):
        from nt2_gb300 import expr as E
        self.torch, self.lib, self.prec, self.E = torch, lib, precision, E
        n = n or 1 << 28
        g = torch.Generator(device=dev).manual_seed(1001)
        self.x = torch.randn(n, device=dev, generator=g)
        self.y = torch.randn(n, device=dev, generator=g)
        X, Y = E.Table(self.x), E.Table(self.y)
        if kind == "sum":
            e, self.shape, op, what = E.exp(X) * Y, (1, n, 1), "sum", f"sum(exp(x)*y) over {n} float32"
        else:
            side = _side(n)
            n = side * side
            e, self.shape, op, what = E.abs_(X - Y), (1, side, side), "sum", \
                f"sum(abs(x - y), 1) of two {side}x{side} float32 tables"
        prog, slots = E.compile_program([], [], fold=e)
        self.prog, self.slots = prog, slots
        self.args = (lib.Arg * len(slots))(*[lib.Arg(t.data_ptr(), 0.0, lib.F32, 0) for t in slots])
        lo, inner, hi = self.shape
        nb = ctypes.c_size_t()
        lib.check(lib.load().nt2g_fold_workspace_size(lo, inner, hi, ctypes.byref(nb)))
        self.ws = torch.empty(max(nb.value, 16), dtype=torch.uint8, device=dev)
        self.out = torch.empty(lo * hi, device=dev)
        self.out64 = torch.empty(lo * hi, dtype=torch.float64, device=dev) if precision != lib.PREC_NT2 else None
        self.op = lib.FOLD[op]
        self.units, self.bytes, self.kernel = n, 8 * n, "fold_inner (run-time compiled)"
        self.launches = 2 if kind == "sum" else 1  # chunk partials, then the in-order combine
        self.name = what + ", one pass through nt2g_eval_fold (no temporary)"

    def step(self, i):
        L = self.lib
        lo, inner, hi = self.shape
        L.check(L.load().nt2g_eval_fold(self.prog.handle, self.args, len(self.slots), lo, inner, hi, self.op, self.prec,
                                        L._ptr(self.ws), self.ws.numel(), L._ptr(self.out), None, L._ptr(self.out64),
                                        L._stream()))


class Rgb2Yuv(Workload):
    SETS = 8
    independent = True

    def __init__(self, torch, lib, dev):
        self.torch, self.lib = torch, lib
        n = 1920 * 1080
        g = torch.Generator(device=dev).manual_seed(1002)
        self.rgb = torch.rand(self.SETS, 3, n, device=dev, generator=g)
        self.yuv = torch.empty_like(self.rgb)
        self.units, self.bytes, self.kernel = n, 24 * n, "k_rgb2yuv"
        self.name = f"rgb2yuv 1920x1080x3 float32 planes, {self.SETS} rotating sets"
        self.flush = f"rotating {self.SETS} sets ({self.SETS * 48} MB)"

    def step(self, i):
        k = i % self.SETS
        r, g, b = self.rgb[k]
        y, u, v = self.yuv[k]
        self.lib.rgb2yuv(r, g, b, y, u, v)


def _side(n):
    """Side of the square table holding about n elements (default 16384)."""
    import math
    return 16384 if not n else max(1, math.isqrt(n))


def make(name, torch, lib, dev, precision, tune=None, n=None):
    if name == "bs":
        return BlackScholes(torch, lib, dev, precision, n)
    if name == "bs_demo":
        return BlackScholesDemo(torch, lib, dev, precision, n)
    if name == "bs_generic":
        return BlackScholesGeneric(torch, lib, dev, precision, mode=1, n=n)
    if name == "bs_interp":
        return BlackScholesGeneric(torch, lib, dev, precision, mode=2, n=n)
    if name in ("reduce", "dot"):
        return Reduce(torch, lib, dev, dot=True)
    if name == "sum":
        return Reduce(torch, lib, dev, dot=False)
    if name == "batched":
        return Batched(torch, lib, dev, per_table=False, precision=precision, tune=tune)
    if name == "pertable":
        return Batched(torch, lib, dev, per_table=True, precision=precision)
    if name == "batched_programs":
        return Batched(torch, lib, dev, per_table=False, precision=precision, tune=tune, programs=True)
    if name == "adjoint":
        return Adjoint(torch, lib, dev)
    if name == "adjoint_fwd":
        return Adjoint(torch, lib, dev, forward_only=True)
    if name in ("adjoint_program", "adjoint_demo"):
        return ProgramAdjoint(torch, lib, dev, "textbook" if name == "adjoint_program" else "demo", precision)
    if name in ("fn_trig", "fn_pow", "fn_gen", "fn_special"):
        return Functors(torch, lib, dev, name[3:], precision, n)
    if name == "sigmadelta":
        return SigmaDelta(torch, lib, dev)
    if name == "rgb2yuv":
        return Rgb2Yuv(torch, lib, dev)
    if name == "sigmadelta_fused":
        return SigmaDeltaFused(torch, lib, dev)
    if name in ("cumsum_col", "cumsum_all", "cummax_row"):
        return Scan(torch, lib, dev, {"cumsum_col": "col", "cumsum_all": "all", "cummax_row": "rowmax"}[name],
                    precision, _side(n))
    if name in ("fold_expr", "fold_expr_col"):
        return FoldExpr(torch, lib, dev, "sum" if name == "fold_expr" else "col", precision, n)
    if name in ("median_col", "median_row", "gmedian"):
        return Median(torch, lib, dev, {"median_col": "col", "median_row": "row", "gmedian": "all"}[name], _side(n))
    if name in ("fold_col", "fold_row", "gmax"):
        return Fold(torch, lib, dev, {"fold_col": "col", "fold_row": "row", "gmax": "max"}[name], precision,
                    _side(n))
    raise SystemExit(f"unknown config {name}")


# ------------------------------------------------------------- CPU baseline
def cpu_baseline(config, budget_s=10.0, inputs=None):
    """NT2's CPU path (the oracle's restatement; NT2 itself needs Boost) on the
    host cores: repeat a bounded sample until budget_s, median rate.  For bs,
    `inputs` (the GPU's rotating set 0) are the options timed, and NT2's
    outputs for them are returned as out["_outputs"] for the bit-exactness
    check of the GPU result."""
    from oracle import oracle
    nthreads = oracle.threads()
    outputs = None
    if config == "bs":
        sample_n = 1 << 20 if inputs is None else inputs[0].size
        f = BlackScholes.cpu(oracle, nthreads, sample_n, inputs)
        what = f"blackscholes call+put on {sample_n} options, OpenMP static over {nthreads} threads"
        outputs = f()
    elif config in ("reduce", "dot", "sum"):
        sample_n = 1 << 26
        rng = np.random.default_rng(1001)
        x = rng.standard_normal(sample_n, dtype=np.float32)
        y = rng.standard_normal(sample_n, dtype=np.float32) if config != "sum" else None
        f = lambda: oracle.sum_plain(x, y, nthreads=nthreads)  # noqa: E731
        what = f"{config} over {sample_n} floats, OpenMP reduction over {nthreads} threads"
    else:
        return None
    def timed(fn, budget):
        fn()
        rates, t_end = [], time.perf_counter() + budget
        while time.perf_counter() < t_end or len(rates) < 3:
            t0 = time.perf_counter()
            fn()
            rates.append(sample_n / (time.perf_counter() - t0))
        return float(np.median(rates)), len(rates)

    value, runs = timed(f, budget_s)
    out = {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
           "sample": what + f", median of {runs} runs"}
    if config == "bs":
        # NT2's own thread rule (shared_memory/transform.hpp: grain = top cache bytes / sizeof(T);
        # n <= 8 grain runs on one thread) and a one-thread figure
        grain = int(oracle.nt2_transform_grain(4))
        nt2_threads = 1 if sample_n <= 8 * grain else nthreads
        one, _ = timed(BlackScholes.cpu(oracle, 1, sample_n, inputs), budget_s / 4)
        out["one_thread"] = one
        out["nt2_rule"] = {"grain": grain, "threads": nt2_threads,
                           "value": one if nt2_threads == 1 else value}
        out["_outputs"] = outputs
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle
    nthreads = oracle.threads()
    if args.config not in ("bs", "reduce", "dot", "sum"):
        print(json.dumps({"impl": "reference", "unavailable": f"no CPU restatement timed for config {args.config}"}))
        return
    if args.config == "bs":
        sample_n = 1 << 20
        rng = np.random.default_rng(1000)
        S = rng.uniform(5, 30, sample_n).astype(np.float32)
        K = rng.uniform(1, 100, sample_n).astype(np.float32)
        T = rng.uniform(0.25, 10, sample_n).astype(np.float32)
        f = lambda: oracle.blackscholes(S, K, T, 0.02, 0.30, nthreads=nthreads)  # noqa: E731
        what = f"blackscholes call+put, {sample_n} options per step (the full batch), {nthreads} OpenMP threads"
        wl_name = f"blackscholes_plain N={sample_n} call+put"
    else:
        sample_n = 1 << 26
        rng = np.random.default_rng(1001)
        x = rng.standard_normal(sample_n, dtype=np.float32)
        y = rng.standard_normal(sample_n, dtype=np.float32) if args.config != "sum" else None
        f = lambda: oracle.sum_plain(x, y, nthreads=nthreads)  # noqa: E731
        what = f"{args.config} over {sample_n} floats per step (2^26 sample of the 2^28 workload), {nthreads} threads"
        wl_name = f"{args.config} n=2^28 float32"
    for _ in range(args.warmup):
        f()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        f()
    dt = time.perf_counter() - t0
    v = sample_n * args.steps / dt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl_name, "implementation": "NT2 CPU path restated in C (oracle/nt2_oracle.c), "
                                                          "NT2 itself needs Boost (absent)"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": what},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


# ------------------------------------------------------------------- GPU arm
def run_ours(args):
    import torch
    import torch.distributed as dist
    from nt2_gb300 import lib
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib.load()
    prec = lib.PREC_NT2 if args.precision == "nt2" else lib.PREC_FAST
    tune = tuple(int(v) for v in args.tune.split(",")) if args.tune else None
    wl = make(args.config, torch, lib, dev, prec, tune, args.n)
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # warm-up (also compiles a generic program's kernel before any capture)
    side = torch.cuda.Stream()
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        for i in range(args.warmup):
            wl.step(i)
    stream.wait_stream(side)
    barrier()
    # The K timed steps are captured once into a CUDA graph and replayed, so
    # the measurement is the device's time for K launches rather than the
    # Python/ctypes cost of issuing them (each launch still happens, in order).
    # Independent steps (disjoint rotating buffer sets) alternate between two
    # streams inside the graph, so one step's tail overlaps the next step's
    # head; steps that share buffers stay in order on one stream.
    graph = None
    n_streams = max(1, args.streams) if wl.independent else 1
    if not args.no_graph:
        graph = torch.cuda.CUDAGraph()
        extra = [torch.cuda.Stream() for _ in range(n_streams - 1)]
        with torch.cuda.graph(graph, stream=side, capture_error_mode="thread_local"):
            fork = torch.cuda.Event()
            fork.record(side)
            for s_ in extra:
                s_.wait_event(fork)
            lanes = [side] + extra
            for i in range(args.steps):
                with torch.cuda.stream(lanes[i % n_streams]):
                    wl.step(i)
            for s_ in extra:
                join = torch.cuda.Event()
                join.record(s_)
                side.wait_event(join)
        barrier()

    def run_k():
        if graph is not None:
            graph.replay()
        else:
            for i in range(args.steps):
                wl.step(i)

    # exactly K steps per trial; trials repeat for ~2 s so the clock sampler
    # sees the load; the median trial is reported
    trials = []
    with ClockSampler(local) as clk:
        t_start = time.perf_counter()
        while True:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            barrier()
            e0.record(stream)
            run_k()
            e1.record(stream)
            barrier()
            trials.append(max_over_ranks(e0.elapsed_time(e1), world, dist, dev))
            if (time.perf_counter() - t_start > args.min_seconds and len(trials) >= 3) or len(trials) >= 100000:
                break
    ms = float(np.median(trials))
    per_step = ms / args.steps
    value = whole_job_value(wl.units, args.steps, world, ms)
    peak, peak_kind = peaks()
    achieved = wl.bytes / (per_step / 1e3) / 1e9
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8" if args.config == "sigmadelta" else "f32",
        "data": "synthetic (seeded, distributions per workload)",
        "config": {"workload": wl.name, "precision": args.precision, "l2": wl.flush,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "trials": len(trials),
                   "launch": (f"CUDA graph of the K steps on {n_streams} stream(s)" if graph is not None else "eager")},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "kernel": wl.kernel,
                     "algorithmic_bytes_per_launch": wl.bytes // wl.launches,
                     "traffic": ncu_traffic(f"{args.config}{'@%d' % args.n if args.n else ''}:{wl.kernel}")},
        "clocks": clk.summary(),
        "gpu_launches": wl.launches * args.steps,
    }
    # end to end through the C ABI with host buffers (where defined)
    if hasattr(wl, "e2e_setup"):
        # K-step trials repeated for at least min_seconds, the median reported
        # (as for the device-resident figure)
        h2d, d2h = wl.e2e_setup()
        for i in range(args.warmup):
            wl.e2e_step(i)
        barrier()
        etrials = []
        t_start = time.perf_counter()
        while True:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for s_ in wl.e2e_streams():
                s_.wait_event(e0)
            for i in range(args.steps):
                wl.e2e_step(i)
            for s_ in wl.e2e_streams():
                done = torch.cuda.Event()
                done.record(s_)
                stream.wait_event(done)
            e1.record(stream)
            barrier()
            etrials.append(max_over_ranks(e0.elapsed_time(e1), world, dist, dev))
            if (time.perf_counter() - t_start > args.min_seconds and len(etrials) >= 3) or len(etrials) >= 100000:
                break
        ems = float(np.median(etrials))
        out["e2e"] = {"value": whole_job_value(wl.units, args.steps, world, ems), "unit": UNIT,
                      "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": ems / args.steps,
                      "trials": len(etrials),
                      "range": [whole_job_value(wl.units, args.steps, world, max(etrials)),
                                whole_job_value(wl.units, args.steps, world, min(etrials))]}
    nt2_out = None
    if rank == 0 and world == 1 and not args.no_cpu:
        inputs = wl.sample()[0] if hasattr(wl, "sample") else None
        cb = cpu_baseline(args.config, budget_s=args.cpu_budget, inputs=inputs)
        if cb is not None:
            nt2_out = cb.pop("_outputs", None)
        out["cpu_baseline"] = cb
    if rank == 0 and getattr(wl, "accuracy", None) is not None:
        out["accuracy"] = wl.accuracy(nt2_out)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--config", default="bs")
    ap.add_argument("--precision", default="fast", choices=["fast", "nt2"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--no-graph", action="store_true", help="issue the K steps eagerly instead of from a graph")
    ap.add_argument("--streams", type=int, default=2, help="streams for independent steps inside the graph")
    ap.add_argument("--tune", default="", help="batched: block_threads,blocks_per_sm,tile_vectors[,vector_width]")
    ap.add_argument("--n", type=int, default=0, help="bs, bs_generic, bs_interp: options per launch (default 2^20); "
                    "fold/scan configs: elements of the square table (default 2^28); fn_*: elements (default 2^26)")
    ap.add_argument("--min-seconds", type=float, default=2.0, help="repeat K-step trials for at least this long")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
