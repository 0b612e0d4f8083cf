"""The allocation-free accumulation entry point against the context one.

lg_accumulate_segments_noalloc is for callers that may not allocate device memory (plug-ins
whose host owns every allocation, real-time loops that must avoid the allocator, fixed
memory budgets): it keeps its binning scratch in a fixed device array shared by all calls.
This checks, through the C ABI, that two calls in a row (the second reusing the array the
first left behind) each produce exactly the fixed-point image lg_accumulate_segments makes
from the same segments, and that a canvas over the array's limit is refused.
"""
import ctypes as C

import numpy as np
import pytest

from light_garden_gb300 import abi, workloads as W

pytestmark = pytest.mark.gpu


def test_noalloc_matches_context_path_twice(gpu):
    import torch
    from light_garden_gb300.runtime import Context

    lib = abi.load()
    pk = W.mid_scene(rays_per_light=1 << 11).packed()
    with Context() as ctx:
        ctx.upload(pk)
        ctx.trace()
        segs = ctx.segments()
        ctx.accumulate_segments(segs)
        ref = ctx.accum()
    assert len(segs) > 1000 and ref.dtype == np.int64
    h, w = pk.params.height, pk.params.width
    d_segs = torch.from_numpy(segs.view(np.uint8).copy()).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        d_acc = torch.full((h * w * 4,), 12345, dtype=torch.int64, device="cuda")  # stale contents
        px = C.c_uint64(0)
        st = lib.lg_accumulate_segments_noalloc(C.c_void_p(d_segs.data_ptr()), len(segs), C.byref(pk.params),
                                                C.c_void_p(d_acc.data_ptr()), C.c_void_p(stream), C.byref(px))
        assert st == abi.LG_OK, (call, abi.STATUS_NAMES.get(st, st))
        torch.cuda.synchronize()
        got = d_acc.cpu().numpy().reshape(h, w, 4)
        assert np.array_equal(got, ref), f"call {call} differs from lg_accumulate_segments"
        assert px.value > 0


def test_noalloc_refuses_canvas_over_limit(gpu):
    import torch

    lib = abi.load()
    p = abi.params_default()
    p.width, p.height = 4096, 4096  # 16384 tiles > 4096
    d_acc = torch.empty(16, dtype=torch.int64, device="cuda")
    st = lib.lg_accumulate_segments_noalloc(None, 0, C.byref(p), C.c_void_p(d_acc.data_ptr()), None, None)
    assert st == abi.LG_ERR_BUDGET
