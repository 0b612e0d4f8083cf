"""Serving with continuous batching (lg_serve_*) on the GPU.

Bar: every request's RGBA16F image is bit-identical to lg_render of the scene alone, whether
it ran alone or among requests admitted before and after it; requests admitted while others
are in flight share launches with them; a step that overflows its ray queue restarts the
requests in flight and their results stay exact.
"""
import numpy as np
import pytest

from light_garden_gb300 import abi, workloads as W

pytestmark = pytest.mark.gpu


def _alone(packed):
    from light_garden_gb300.runtime import Context
    with Context() as c:
        c.upload(packed)
        img, _ = c.render()
    return img


def _scenes(seed, n, scale=1 / 128):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        w = W.batch_scene(rng)
        w.params.width = min(w.params.width, 512)
        w.params.height = min(w.params.height, 512)
        out.append(W.scale_rays(w, scale).packed())
    return out


def _drain(ctx, ids, extra=None, max_steps=5000):
    """Steps until every id is polled; extra: {step number: [scenes to submit then]}."""
    got, log = {}, []
    pending = set(ids)
    for k in range(max_steps):
        if extra and k in extra:
            for sc in extra[k]:
                rid = ctx.serve_submit(sc)
                pending.add(rid)
                ids.append(rid)
        st = ctx.serve_step()
        log.append(st)
        for rid in list(pending):
            img = ctx.serve_poll(rid)
            if img is not None:
                got[rid] = img
                pending.discard(rid)
        if not pending and not (extra and any(s > k for s in extra)):
            break
    return got, log


def test_serve_results_equal_alone_with_arrivals_in_flight(ctx):
    first, later = _scenes(21, 4), _scenes(22, 4)
    ctx.serve_begin(hbm_budget_bytes=4 << 30, max_slots=64)
    ids = [ctx.serve_submit(sc) for sc in first]
    got, log = _drain(ctx, ids, extra={2: later[:2], 5: later[2:]})
    scenes = first + later
    assert len(got) == len(scenes)
    for rid, sc in zip(ids, scenes):
        assert np.array_equal(got[rid], _alone(sc)), f"request {rid}"
    # continuous batching: some step admitted new work while older requests were in flight
    assert any(s["admitted"] > 0 and s["in_flight"] > s["admitted"] for s in log)
    ctx.serve_end()


def test_serve_small_queue_restarts_stay_exact(ctx):
    # The mid scene with 2 048 primaries peaks at about 5.4 live rays per primary (generation
    # 12).  A 6 MB budget gives a ray queue of about 6 600 rays: the step that outgrows it
    # restarts the request with a queue twice as large, and the result stays exact.
    scenes = [W.mid_scene(rays_per_light=1 << 8).packed(), W.plain_small(accum=abi.LG_ACCUM_FIXED64, num_rays=2048).packed()]
    for sc in scenes:
        sc.params.width, sc.params.height = 256, 192
    ctx.serve_begin(hbm_budget_bytes=6 << 20, max_slots=4)
    ids = [ctx.serve_submit(sc) for sc in scenes]
    got, log = _drain(ctx, ids)
    for rid, sc in zip(ids, scenes):
        assert np.array_equal(got[rid], _alone(sc))
    assert sum(s["restarted"] for s in log) >= 1
    ctx.serve_end()


def test_serve_errors(ctx):
    sc = W.plain_small(accum=abi.LG_ACCUM_FIXED64).packed()
    with pytest.raises(abi.LgError) as e:
        ctx.serve_submit(sc)
    assert e.value.status == abi.LG_ERR_NO_SCENE
    ctx.serve_begin(hbm_budget_bytes=64 << 20, max_slots=8)
    with pytest.raises(abi.LgError) as e:
        ctx.upload(sc)
    assert e.value.status == abi.LG_ERR_INVALID_ARGUMENT
    f32 = W.plain_small(accum=abi.LG_ACCUM_F32).packed()
    with pytest.raises(abi.LgError) as e:
        ctx.serve_submit(f32)
    assert e.value.status == abi.LG_ERR_UNSUPPORTED
    huge = W.mid_scene().packed()  # 2 M primaries: more than a 64 MB budget's queue
    with pytest.raises(abi.LgError) as e:
        ctx.serve_submit(huge)
    assert e.value.status == abi.LG_ERR_BUDGET
    ctx.serve_shapes[12345] = (1, 1)
    with pytest.raises(abi.LgError) as e:
        ctx.serve_poll(12345)
    assert e.value.status == abi.LG_ERR_NOT_FOUND
    rid = ctx.serve_submit(sc)
    assert ctx.serve_poll(rid) is None  # queued, not run yet
    got, _ = _drain(ctx, [rid])
    assert np.array_equal(got[rid], _alone(sc))
    ctx.serve_end()
    ctx.upload(sc)  # the single-scene path works again
    img, _ = ctx.render()
    assert np.array_equal(img, _alone(sc))
