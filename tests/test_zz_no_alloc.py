"""The allocation-free reduction entry point, nt2g_reduce_f32_noalloc, for
callers that cannot allocate device memory (a host runtime that owns every
device allocation, code that must not let cudaMalloc/cudaFree synchronize
the device, wrappers with nowhere to keep a workspace).  Its scratch is a
static device array inside the library instead of a caller workspace; the
results must match the workspace entry point, nt2g_reduce_f32, on the same
inputs.  Two calls in a row check that the shared array is reset between
calls.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _noalloc(lib, x, y=None):
    o64 = torch.zeros(1, dtype=torch.float64, device=x.device)
    o32 = torch.zeros(1, dtype=torch.float32, device=x.device)
    st = lib.load().nt2g_reduce_f32_noalloc(ctypes.c_void_p(x.data_ptr()),
                                             None if y is None else ctypes.c_void_p(y.data_ptr()),
                                             x.numel(), ctypes.c_void_p(o64.data_ptr()),
                                             ctypes.c_void_p(o32.data_ptr()), lib._stream())
    lib.check(st)
    torch.cuda.synchronize()
    return float(o64.item()), float(o32.item())


def test_noalloc_reduction_matches_workspace_entry_point(lib, dev):
    red = lib.Reducer(dev)
    rng = np.random.default_rng(2024)
    for n in ((1 << 24) + 3, 100003):  # two calls in a row through the shared static scratch
        x = torch.from_numpy(rng.standard_normal(n, dtype=np.float32)).to(dev)
        y = torch.from_numpy(rng.standard_normal(n, dtype=np.float32)).to(dev)
        for yy in (None, y):
            r64, r32 = red(x, yy)
            torch.cuda.synchronize()
            g64, g32 = _noalloc(lib, x, yy)
            assert g64 == pytest.approx(float(r64.item()), rel=1e-12)
            assert g32 == pytest.approx(float(r32.item()), rel=1e-6)
