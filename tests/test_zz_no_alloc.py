"""rt_trace_noalloc: ray queries for callers that cannot allocate device memory.

Some host applications own all of the device's memory through their own pool,
or trace from a loop that must not stall on cudaMalloc.  rt_trace_noalloc
keeps its only scratch (the ray-queue counter) in a static device array
instead of the per-stream cudaMalloc workspace that rt_trace creates.  This
test calls it through the C ABI, first, on a stream the library has never
seen, and checks that the library's workspace count does not grow (no
cudaMalloc); then it checks each of two calls in a row, for closest hit, any
hit and the Moller-Trumbore mode, against rt_trace bit for bit (the tolerance
every trace test here uses), and the size limit.  It sits in a file of its own
that pytest collects last.
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


FLAGS = [(0, {}), (1, {"any_hit": True}), (4, {"mt": True})]  # RT_TRACE_ANY = 1, RT_TRACE_MT = 4


def test_noalloc_matches_rt_trace(rt, cuda):
    f = noalloc_fn(rt)
    tris = rt.gen_soup(17, 0, 120_000, 1.0, 0.004)
    rays = rt.gen_rays(17, 0, 500_000, 1.0, 1e-4, float("inf"))
    n = len(rays)
    with rt.Scene(tris) as sc:
        d_rays = cuda.from_numpy(rays.view(np.uint8)).cuda()
        outs = {flag: [cuda.full((n * 8,), 0xCD, dtype=cuda.uint8, device="cuda") for _ in range(2)]
                for flag, _ in FLAGS}
        side = cuda.cuda.Stream()  # a stream no library call has used
        cuda.cuda.synchronize()
        before = rt.workspace_count()
        for flag, _ in FLAGS:
            for call in range(2):
                st = f(sc.handle, d_rays.data_ptr(), n, outs[flag][call].data_ptr(), flag, side.cuda_stream)
                assert st == 0, rt.lib().rt_last_error_string()
        side.synchronize()
        assert rt.workspace_count() == before, "rt_trace_noalloc created a device workspace"
        for flag, kw in FLAGS:
            ref = cuda.empty(n * 8, dtype=cuda.uint8, device="cuda")
            sc.trace(d_rays, ref, **kw)
            cuda.cuda.synchronize()
            ref_h = ref.cpu().numpy().view(rt.HIT_DTYPE)
            assert (ref_h["prim"] != rt.NO_HIT).sum() > n // 10
            for call in range(2):
                got = outs[flag][call].cpu().numpy().view(rt.HIT_DTYPE)
                assert np.array_equal(got.view(np.uint64), ref_h.view(np.uint64)), f"flags {flag} call {call} differs"
        # beyond the scratch counter's range: a clear error, nothing launched
        st = f(sc.handle, d_rays.data_ptr(), 0x80000001, d_rays.data_ptr(), 0, side.cuda_stream)
        assert st == 1
        assert b"maximum" in rt.lib().rt_last_error_string()
