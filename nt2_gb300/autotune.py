"""Batched-launch tuning with a JSON cache.

``tuned(items, precision)`` returns the fastest ``BatchTune`` (block size,
resident blocks per SM or static striding, float4 vectors per thread per
tile, float4 vectors in flight per thread) for a batch shape on the current
GPU, measuring with ``nt2g_batch_autotune`` the first
time and reading the cache afterwards.  The key is the GPU name, the
precision, the expression mix and the table-size histogram (log2 buckets), so
batches of the same shape share one entry.  Cache file: $NT2G_TUNE_CACHE, or
~/.cache/nt2g/batch_tune.json.
"""
import ctypes
import json
import os

import numpy as np

from . import lib


def cache_path():
    return os.environ.get("NT2G_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "nt2g",
                                                          "batch_tune.json"))


def shape_key(items, precision):
    import torch
    sizes = np.array([it.n for it in items], np.int64)
    exprs = np.array([it.expr for it in items], np.int64)
    hist = np.bincount(np.log2(np.maximum(sizes, 1)).astype(np.int64), minlength=32)
    mix = np.bincount(exprs, minlength=4)
    return json.dumps([torch.cuda.get_device_name(), int(precision), mix.tolist(), hist.tolist()])


def tuned(items, precision=lib.PREC_FAST, reps=3, stream=None):
    path = cache_path()
    key = shape_key(items, precision)
    cache = {}
    if os.path.exists(path):
        try:
            cache = json.load(open(path))
        except (OSError, ValueError):
            cache = {}
    if key in cache:
        t = cache[key]["tune"]
        vw = t[3] if len(t) > 3 else 1
        return lib.BatchTune(t[0], t[1], t[2], precision, vw), cache[key]["ms"], True
    best, ms = lib.BatchTune(), ctypes.c_float()
    lib.check(lib.load().nt2g_batch_autotune(items, len(items), None, 0, reps, precision, lib._stream(stream),
                                             ctypes.byref(best), ctypes.byref(ms)))
    cache[key] = {"tune": [best.block_threads, best.blocks_per_sm, best.tile_vectors, best.vector_width],
                  "ms": ms.value}
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        json.dump(cache, f, indent=1)
    return best, ms.value, False
