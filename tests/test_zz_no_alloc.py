"""rt_trace_noalloc: ray queries for callers that cannot allocate device memory.

Some host applications own all of the device's memory through their own pool,
or trace from a loop that must not stall on cudaMalloc.  rt_trace_noalloc
keeps its only scratch (the ray-queue counter) in a static device array
instead of a per-stream cudaMalloc workspace.  This test calls it through the
C ABI twice in a row and checks each result against rt_trace bit for bit
(the tolerance every trace test here uses), and checks the size limit.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def noalloc_fn(rt):
    f = rt.lib().rt_trace_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p]
    return f


def test_noalloc_matches_rt_trace(rt, cuda):
    f = noalloc_fn(rt)
    tris = rt.gen_soup(17, 0, 120_000, 1.0, 0.004)
    rays = rt.gen_rays(17, 0, 500_000, 1.0, 1e-4, float("inf"))
    n = len(rays)
    stream = cuda.cuda.current_stream().cuda_stream or None
    with rt.Scene(tris) as sc:
        d_rays = cuda.from_numpy(rays.view(np.uint8)).cuda()
        for any_hit in (False, True):
            ref = cuda.empty(n * 8, dtype=cuda.uint8, device="cuda")
            sc.trace(d_rays, ref, any_hit=any_hit)
            cuda.cuda.synchronize()
            ref_h = ref.cpu().numpy().view(rt.HIT_DTYPE)
            for call in range(2):
                out = cuda.full((n * 8,), 0xCD, dtype=cuda.uint8, device="cuda")
                st = f(sc.handle, d_rays.data_ptr(), n, out.data_ptr(), 1 if any_hit else 0, stream)
                assert st == 0, rt.lib().rt_last_error_string()
                cuda.cuda.synchronize()
                got = out.cpu().numpy().view(rt.HIT_DTYPE)
                assert np.array_equal(got.view(np.uint64), ref_h.view(np.uint64)), f"call {call} differs"
        assert (ref_h["prim"] != rt.NO_HIT).sum() > n // 10
        # beyond the scratch counter's range: a clear error, nothing launched
        st = f(sc.handle, d_rays.data_ptr(), 0x80000001, d_rays.data_ptr(), 0, stream)
        assert st == 1
        assert b"maximum" in rt.lib().rt_last_error_string()
