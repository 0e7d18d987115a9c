"""Batched persistent launch over uneven tables: every table's result is
bit-identical to the plain kernel on that table, through the persistent
kernel (dynamic and static tile schedules), the per-table launches and the
CUDA-graph replay."""
import ctypes

import numpy as np
import pytest
import torch

from helpers import batched_sizes

pytestmark = pytest.mark.gpu


def _make(lib, dev, sizes, exprs, seed=1003):
    rng = np.random.default_rng(seed)
    tabs = []
    for n, ex in zip(sizes, exprs):
        n = int(n)
        if ex == lib.BATCH_BLACKSCHOLES:
            ins = [rng.uniform(5, 30, n), rng.uniform(1, 100, n), rng.uniform(0.25, 10, n)]
            s = (0.3, 0.02)
        elif ex == lib.BATCH_SAXPY:
            ins = [rng.standard_normal(n)]
            s = (float(np.float32(rng.uniform(-2, 2))), 0.0)
        else:
            ins = [rng.standard_normal(n) for _ in range(3)]
            s = (0.0, 0.0)
        ins = [torch.from_numpy(a.astype(np.float32)).to(dev) for a in ins]
        y0 = torch.from_numpy(rng.standard_normal(n).astype(np.float32)).to(dev) if ex == lib.BATCH_SAXPY else None
        tabs.append((int(ex), n, ins, s, y0))
    return tabs


def _items(lib, tabs, outs):
    items = (lib.BatchItem * len(tabs))()
    for i, ((ex, n, ins, s, _), o) in enumerate(zip(tabs, outs)):
        items[i].expr, items[i].n = ex, n
        for j, t in enumerate(ins):
            items[i].inp[j] = t.data_ptr()
        for j, t in enumerate(o):
            items[i].out[j] = t.data_ptr()
        items[i].s[0], items[i].s[1] = s
    return items


def _fresh_outs(lib, tabs):
    outs = []
    for ex, n, ins, s, y0 in tabs:
        if ex == lib.BATCH_BLACKSCHOLES:
            outs.append([torch.zeros_like(ins[0]), torch.zeros_like(ins[0])])
        elif ex == lib.BATCH_SAXPY:
            outs.append([y0.clone()])
        else:
            outs.append([torch.zeros_like(ins[0])])
    return outs


def _reference(lib, tabs):
    ref = []
    for ex, n, ins, s, y0 in tabs:
        if ex == lib.BATCH_BLACKSCHOLES:
            c, p = torch.empty_like(ins[0]), torch.empty_like(ins[0])
            lib.blackscholes(ins[0], ins[1], ins[2], c, p, s[1], sigma_s=s[0])
            ref.append([c, p])
        elif ex == lib.BATCH_SAXPY:
            y = y0.clone()
            lib.saxpy(s[0], ins[0], y)
            ref.append([y])
        else:
            o = torch.empty_like(ins[0])
            lib.expr3(ins[0], ins[1], ins[2], o)
            ref.append([o])
    torch.cuda.synchronize()
    return ref


def _check(outs, ref):
    for k, (o, r) in enumerate(zip(outs, ref)):
        for a, b in zip(o, r):
            assert torch.equal(a.view(torch.int32), b.view(torch.int32)), k


@pytest.mark.parametrize("tune", [(256, 0, 4), (128, 0, 1), (512, -1, 2), (256, 2, 8)],
                         ids=["dyn256x4", "dyn128x1", "static512x2", "dyn256x8_2perSM"])
def test_batched_matches_plain_kernels(lib, dev, tune):
    sizes, exprs = batched_sizes(count=96, lo=1, hi=300000, seed=5)
    sizes[:3] = [1, 3, 5]
    tabs = _make(lib, dev, sizes, exprs)
    ref = _reference(lib, tabs)
    L = lib.load()
    t = lib.BatchTune(tune[0], tune[1], tune[2], lib.PREC_FAST)
    stream = torch.cuda.Stream()
    for mode in ("run", "per_table", "graph"):
        outs = _fresh_outs(lib, tabs)
        items = _items(lib, tabs, outs)
        h = ctypes.c_void_p()
        lib.check(L.nt2g_batch_create(items, len(tabs), ctypes.byref(t), ctypes.byref(h)))
        try:
            fn = dict(run=L.nt2g_batch_run, per_table=L.nt2g_batch_run_per_table, graph=L.nt2g_batch_run_graph)[mode]
            torch.cuda.synchronize()
            lib.check(fn(h, ctypes.c_void_p(stream.cuda_stream)))
            stream.synchronize()
            _check(outs, ref)
            if mode == "graph":  # replay: reset the in-place saxpy outputs first
                for (ex, n, ins, s, y0), o in zip(tabs, outs):
                    if ex == lib.BATCH_SAXPY:
                        o[0].copy_(y0)
                torch.cuda.synchronize()
                lib.check(fn(h, ctypes.c_void_p(stream.cuda_stream)))
                stream.synchronize()
                _check(outs, ref)
            el, by = ctypes.c_int64(), ctypes.c_int64()
            lib.check(L.nt2g_batch_stats(h, ctypes.byref(el), ctypes.byref(by)))
            assert el.value == int(np.sum(sizes))
        finally:
            L.nt2g_batch_destroy(h)


@pytest.mark.parametrize("prec", ["nt2", "fast"])
def test_batched_against_oracle(lib, dev, oracle, prec):
    """The first 256 tables of the benchmark's own 4096-table mix (seed 1003:
    sizes log-uniform in [1024, 4194304], ~1.3e8 elements, the three
    expressions interleaved) through one persistent launch, checked against
    the oracle rather than against this library's plain kernels:
      NT2 policy: every table bit-identical to the CPU restatement of NT2's
        evaluation (Black-Scholes, saxpy, expr3);
      fast policy: saxpy bit-identical (it is NT2's arithmetic), expr3 within
        4 ulp of FP64, Black-Scholes within the stated conditioned-ulp bound
        (max, p99.9, mean) and no worse than NT2's own float evaluation of the
        same options (max)."""
    from helpers import BS_FAST_MAX, BS_FAST_MEAN, BS_FAST_P999, F32, conditioned_ulp, std_ulp
    sizes, exprs = batched_sizes()
    sizes, exprs = sizes[:256], exprs[:256]
    p = lib.PREC_NT2 if prec == "nt2" else lib.PREC_FAST
    tabs = _make(lib, dev, sizes, exprs)
    outs = _fresh_outs(lib, tabs)
    items = _items(lib, tabs, outs)
    L = lib.load()
    t = lib.BatchTune(256, 0, 16, p)
    h = ctypes.c_void_p()
    lib.check(L.nt2g_batch_create(items, len(tabs), ctypes.byref(t), ctypes.byref(h)))
    try:
        torch.cuda.synchronize()
        lib.check(L.nt2g_batch_run(h, lib._stream()))
        torch.cuda.synchronize()
    finally:
        L.nt2g_batch_destroy(h)
    bs_in, bs_out, bs_ref = [], [], []
    for k, ((ex, n, ins, s, y0), o) in enumerate(zip(tabs, outs)):
        a = [x.cpu().numpy() for x in ins]
        got = [x.cpu().numpy() for x in o]
        if ex == lib.BATCH_SAXPY:
            ref = oracle.saxpy(np.float32(s[0]), a[0], y0.cpu().numpy())
            assert np.array_equal(got[0].view(np.uint32), np.asarray(ref, F32).view(np.uint32)), k
        elif ex == lib.BATCH_EXPR3:
            if p == lib.PREC_NT2:
                assert np.array_equal(got[0].view(np.uint32), oracle.expr3(*a).view(np.uint32)), k
            else:
                e = std_ulp(got[0], oracle.expr3_f64(*a))
                assert e.max() <= 4.0, (k, e.max())
        else:
            if p == lib.PREC_NT2:
                rc, rp = oracle.blackscholes(a[0], a[1], a[2], s[1], s[0])
                assert np.array_equal(got[0].view(np.uint32), rc.view(np.uint32)), k
                assert np.array_equal(got[1].view(np.uint32), rp.view(np.uint32)), k
            else:
                bs_in.append(a)
                bs_out.append(got)
    if p == lib.PREC_FAST:
        S, K, T = (np.concatenate([a[j] for a in bs_in]) for j in range(3))
        c, pp = (np.concatenate([g[j] for g in bs_out]) for j in range(2))
        c64, p64, terms = oracle.blackscholes_f64(S, K, T, 0.02, 0.3)
        rc, rp = oracle.blackscholes(S, K, T, 0.02, 0.3)
        fl = 2.0 ** -102
        sc = np.maximum(np.maximum(np.abs(terms[:, 0]), np.abs(terms[:, 1])), fl)
        sp = np.maximum(np.maximum(np.abs(terms[:, 2]), np.abs(terms[:, 3])), fl)
        for got, ref64, scale, nt2 in ((c, c64, sc, rc), (pp, p64, sp, rp)):
            e, en = conditioned_ulp(got, ref64, scale), conditioned_ulp(nt2, ref64, scale)
            q = lambda v: np.quantile(v, 0.999)  # noqa: E731
            print(f"\nbatched fast BS ({S.size} options): max {e.max():.2f} mean {e.mean():.3f} p99.9 {q(e):.2f}; "
                  f"NT2's own: max {en.max():.2f} mean {en.mean():.3f} p99.9 {q(en):.2f}")
            assert e.max() <= BS_FAST_MAX and e.max() <= en.max()
            assert q(e) <= BS_FAST_P999 and e.mean() <= BS_FAST_MEAN


def test_autotuner_picks_a_candidate_and_caches(lib, dev, tmp_path, monkeypatch):
    from nt2_gb300 import autotune
    monkeypatch.setenv("NT2G_TUNE_CACHE", str(tmp_path / "tune.json"))
    sizes, exprs = batched_sizes(count=64, lo=1000, hi=200000, seed=6)
    tabs = _make(lib, dev, sizes, exprs)
    items = _items(lib, tabs, _fresh_outs(lib, tabs))
    best, ms, cached = autotune.tuned(items, lib.PREC_FAST, reps=2)
    assert not cached and ms > 0 and best.block_threads in (128, 256, 512)
    best2, ms2, cached2 = autotune.tuned(items, lib.PREC_FAST)
    assert cached2 and (best2.block_threads, best2.tile_vectors) == (best.block_threads, best.tile_vectors)
    # a run with the chosen tune is bit-identical to the plain kernels
    ref = _reference(lib, tabs)
    outs = _fresh_outs(lib, tabs)
    h = ctypes.c_void_p()
    L = lib.load()
    lib.check(L.nt2g_batch_create(_items(lib, tabs, outs), len(tabs), ctypes.byref(best), ctypes.byref(h)))
    try:
        lib.check(L.nt2g_batch_run(h, lib._stream()))
        torch.cuda.synchronize()
        _check(outs, ref)
    finally:
        L.nt2g_batch_destroy(h)
