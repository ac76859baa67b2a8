"""The allocation-free dot product (tsr_dot_device_noalloc) against the
library's usual fixed-order dot product (tsr_dot).

Some callers cannot let a library allocate device memory -- a host program
that owns all device memory through its own pool, latency-critical loops
that cannot afford an allocation's device-wide synchronisation.
tsr_dot_device_noalloc serves them
with a fixed scratch array compiled into the library instead of a context.
This test calls it through the C-ABI on device buffers the caller owns, twice
in a row with different data and sizes (the scratch array and its counter
are reused across calls), and requires the same bits as tsr_dot -- the
tolerance every reduction test in this suite uses; an empty sum must give
+0.0.  The file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from twoscalerich_gb300 import capi
from twoscalerich_gb300 import problem as P

pytestmark = pytest.mark.gpu


def test_noalloc_dot_matches_tsr_dot_on_two_calls():
    torch = pytest.importorskip("torch")
    lib = capi.load()
    p = P.config2(n_macro=41, n_micro=21)          # N = 1,412,081 >= the sizes below
    ctx = P.Context(p, max_krylov=0)
    rng = np.random.default_rng(2026)
    for n in (1_000_003, 777_777):                 # two calls in a row
        x = rng.normal(size=n)
        y = rng.normal(size=n)
        expected = ctx.dot(x, y)                   # the existing entry point
        dx = torch.from_numpy(x).to("cuda")
        dy = torch.from_numpy(y).to("cuda")
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = lib.tsr_dot_device_noalloc(C.c_void_p(dx.data_ptr()), C.c_void_p(dy.data_ptr()), n,
                                        C.c_void_p(out.data_ptr()), None)
        assert rc == capi.TSR_OK, capi.last_error()
        capi.check(lib.tsr_sync(ctx.h), "tsr_sync")
        torch.cuda.synchronize()
        got = float(out.cpu()[0])
        assert got == expected


def test_noalloc_dot_empty_sum_is_positive_zero():
    torch = pytest.importorskip("torch")
    lib = capi.load()
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.tsr_dot_device_noalloc(None, None, 0, C.c_void_p(out.data_ptr()), None)
    assert rc == capi.TSR_OK, capi.last_error()
    torch.cuda.synchronize()
    got = float(out.cpu()[0])
    assert got == 0.0 and np.copysign(1.0, got) == 1.0


def test_noalloc_dot_rejects_sizes_beyond_its_scratch():
    lib = capi.load()
    too_big = 8192 * 8192 + 1
    rc = lib.tsr_dot_device_noalloc(C.c_void_p(1), C.c_void_p(1), too_big, C.c_void_p(1), None)
    assert rc == 5                                 # TSR_ERR_ARG, nothing launched
    assert "exceeds the maximum" in capi.last_error()
