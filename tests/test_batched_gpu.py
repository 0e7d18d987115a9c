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
