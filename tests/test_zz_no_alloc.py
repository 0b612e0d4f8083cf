"""The allocation-free accumulation entry point against the context one.

lg_accumulate_segments_noalloc is for callers that may not allocate device memory (plug-ins
whose host owns every allocation, real-time loops that must avoid the allocator, fixed
memory budgets): it keeps its binning scratch in a fixed device array shared by all calls.
This checks, through the C ABI, that two calls in a row (the second reusing the array the
first left behind) each produce exactly the fixed-point image lg_accumulate_segments makes
from the same segments, in the additive, min/max and FP32 raster modes; that a canvas over
the array's limit is refused; and that a call with more (segment, tile) pairs than the
array holds returns LG_ERR_BUDGET and leaves the array fit for the next call.
"""
import ctypes as C

import numpy as np
import pytest

from light_garden_gb300 import abi, workloads as W

pytestmark = pytest.mark.gpu


def _mid_segments():
    from light_garden_gb300.runtime import Context

    pk = W.mid_scene(rays_per_light=1 << 11).packed()
    with Context() as ctx:
        ctx.upload(pk)
        ctx.trace()
        segs = ctx.segments()
    assert len(segs) > 1000
    return pk, segs


def _context_image(params, segs):
    """lg_accumulate_segments of a context: the image the allocation-free call must match."""
    from light_garden_gb300.runtime import Context

    pk = W.plain_small().packed()
    pk.params = params
    with Context() as ctx:
        ctx.upload(pk)
        ctx.accumulate_segments(segs)
        return ctx.accum()


def _noalloc(lib, params, d_segs, n, d_acc):
    import torch

    px = C.c_uint64(0)
    stream = torch.cuda.current_stream().cuda_stream
    st = lib.lg_accumulate_segments_noalloc(C.c_void_p(d_segs.data_ptr()) if n else None, n, C.byref(params),
                                            C.c_void_p(d_acc.data_ptr()), C.c_void_p(stream), C.byref(px))
    torch.cuda.synchronize()
    return st, px.value


def _blend(mode):
    """params of one of the raster modes the entry point dispatches to"""
    p = abi.params_default()
    if mode == "f32":
        p.accum = abi.LG_ACCUM_F32
    elif mode == "minmax":
        p.color_blend.src_factor, p.color_blend.dst_factor, p.color_blend.op = abi.LG_BF_ONE, abi.LG_BF_ONE, abi.LG_BO_MAX
        p.alpha_blend.src_factor, p.alpha_blend.dst_factor, p.alpha_blend.op = abi.LG_BF_ONE, abi.LG_BF_ONE, abi.LG_BO_MIN
    return p


@pytest.mark.parametrize("mode", ["add", "minmax", "f32"])
def test_noalloc_matches_context_path_twice(gpu, mode):
    import torch

    lib = abi.load()
    pk, segs = _mid_segments()
    p = _blend(mode)
    p.width, p.height = pk.params.width, pk.params.height
    ref = _context_image(p, segs)
    h, w = p.height, p.width
    d_segs = torch.from_numpy(segs.view(np.uint8).copy()).cuda()
    dt = torch.float32 if mode == "f32" else torch.int64
    for call in range(2):
        d_acc = torch.full((h * w * 4,), 12345, dtype=dt, device="cuda")  # stale contents
        st, px = _noalloc(lib, p, d_segs, len(segs), d_acc)
        assert st == abi.LG_OK, (call, abi.STATUS_NAMES.get(st, st))
        got = d_acc.cpu().numpy().reshape(h, w, 4)
        if mode == "f32":
            # FP32 atomics add in no fixed order.  Every colour term is >= 0 and each segment
            # adds alpha^2 = 1, so the alpha channel counts a pixel's n terms exactly (from the
            # clear value 1): two orders of the same n-term sum differ by at most 2 n u |sum|
            assert np.array_equal(got[..., 3], ref[..., 3])
            n = ref[..., 3:4].astype(np.float64)
            tol = 2.0 * n * 2.0 ** -24 * np.abs(ref.astype(np.float64)) + 1e-30
            diff = np.abs(got.astype(np.float64) - ref)
            assert (diff <= tol).all(), f"call {call}: worst excess {(diff / tol).max():.3g} x the summation bound"
        else:
            assert np.array_equal(got, ref), f"call {call} differs from lg_accumulate_segments"
        assert px > 0


def test_noalloc_budget_overflow_then_recovers(gpu):
    """Diagonals across a 2048x2048 canvas cross ~127 tiles each: 70,000 of them need about
    8.9 M (segment, tile) pairs, more than the array holds (8,000,000)."""
    import torch

    lib = abi.load()
    rng = np.random.default_rng(5)
    n = 70000
    big = np.zeros(n, dtype=abi.segment_dtype())
    j = rng.uniform(-0.02, 0.02, (n, 2)).astype(np.float32)
    big["x0"], big["y0"] = -0.99 + j[:, 0], -0.99 + j[:, 1]
    big["x1"], big["y1"] = 0.99 - j[:, 1], 0.99 - j[:, 0]
    big["color"] = np.float32(0.25)
    p = abi.params_default()
    p.width, p.height = 2048, 2048
    d_big = torch.from_numpy(big.view(np.uint8).copy()).cuda()
    d_acc = torch.zeros(2048 * 2048 * 4, dtype=torch.int64, device="cuda")
    st, _ = _noalloc(lib, p, d_big, n, d_acc)
    assert st == abi.LG_ERR_BUDGET, abi.STATUS_NAMES.get(st, st)
    # the next call starts from a clean array: a small frame matches the context path again
    small = big[:500]
    ref = _context_image(p, small)
    d_small = torch.from_numpy(small.view(np.uint8).copy()).cuda()
    st, _ = _noalloc(lib, p, d_small, len(small), d_acc)
    assert st == abi.LG_OK
    assert np.array_equal(d_acc.cpu().numpy().reshape(2048, 2048, 4), ref)


def test_noalloc_refuses_canvas_over_limit(gpu):
    import torch

    lib = abi.load()
    p = abi.params_default()
    p.width, p.height = 4096, 4096  # 16384 tiles > 4096
    d_acc = torch.empty(16, dtype=torch.int64, device="cuda")
    st = lib.lg_accumulate_segments_noalloc(None, 0, C.byref(p), C.c_void_p(d_acc.data_ptr()), None, None)
    assert st == abi.LG_ERR_BUDGET
    # within the tile limit but wider than a context accepts (32768 pixels per side)
    p.width, p.height = 131072, 32
    st = lib.lg_accumulate_segments_noalloc(None, 0, C.byref(p), C.c_void_p(d_acc.data_ptr()), None, None)
    assert st == abi.LG_ERR_INVALID_ARGUMENT
