"""The committed golden fixtures (``tests/golden``, written by ``make_golden.py``).

CPU: the oracle reproduces every fixture bit for bit (segments, path records, FP64 endpoints,
image digests), so the checker itself cannot drift.  GPU: the CUDA path, traced at the
workload's full size, matches the stored subset under the parity rules of ``parity.py``, and
its fixed-point image of the stored segments has the stored digest.
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from light_garden_gb300 import abi, workloads as W
from parity import compare

GOLD = Path(__file__).resolve().parent / "golden"
INDEX = json.loads((GOLD / "golden.json").read_text())


def load(name):
    z = np.load(GOLD / f"{name}.npz")
    return z["segs"], z["paths"], z["s64"]


def load_chords(name):
    return np.load(GOLD / f"{name}.npz")["chords"]


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", sorted(INDEX))
def test_oracle_reproduces_fixture(oracle, name):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", GOLD / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    segs, paths, s64, chords, meta = mg.run_case(name)
    gs, gp, g64 = load(name)
    assert meta == INDEX[name]
    assert segs.tobytes() == gs.tobytes()
    assert paths.tobytes() == gp.tobytes()
    assert s64.tobytes() == g64.tobytes()
    assert chords.tobytes() == load_chords(name).tobytes()


def test_fixture_invariants():
    """Properties any correct trace has, checked on the stored data."""
    for name in INDEX:
        segs, paths, s64 = load(name)
        tr = paths["source"] == abi.LG_SRC_TRACE
        # f32 endpoints are the rounded FP64 ones
        assert (segs["x0"] == s64[:, 0].astype(np.float32)).all()
        assert (segs["y1"] == s64[:, 3].astype(np.float32)).all()
        # alpha is never split by a bounce (tracer.rs:454-471) and colours stay in [0, 1]
        c = np.stack([segs["color"][:, i] for i in range(4)], 1)
        assert (c >= 0).all() and (c <= 1).all()
        # every non-primary segment starts where its parent ended
        key = {(int(q["light"]), int(q["primary"]), int(q["gen"]), int(q["path"])): i
               for i, q in enumerate(paths) if q["source"] == abi.LG_SRC_TRACE}
        for i in np.nonzero(tr & (paths["gen"] > 0))[0][:2000]:
            q = paths[i]
            g = int(q["gen"])
            parent = (int(q["light"]), int(q["primary"]), g - 1, int(q["path"]) & ((1 << (g - 1)) - 1))
            if parent in key:
                j = key[parent]
                assert s64[i, 0] == s64[j, 2] and s64[i, 1] == s64[j, 3]


# ---- GPU ------------------------------------------------------------------------------------
@pytest.mark.gpu
def test_gpu_plain_small_matches_fixture(ctx):
    segs, paths, s64 = load("plain_small_fixed64")
    pk = W.plain_small(accum=abi.LG_ACCUM_FIXED64).packed()
    pk.params.record_paths = 1
    ctx.upload(pk)
    st = ctx.trace()
    g_segs, g_paths = ctx.segments(paths=True)
    rep = compare(g_segs, g_paths, segs, paths, s64)
    assert rep.ok(), rep
    assert rep.matched > 0.99 * len(segs)
    # the GPU raster of the stored segments reproduces the stored image digests
    ctx.accumulate_segments(segs)
    acc = ctx.accum()
    meta = INDEX["plain_small_fixed64"]
    assert digest(acc) == meta["accum_sha256"]
    assert digest(ctx.resolve_f16()) == meta["f16_sha256"]
    assert digest(ctx.resolve_rgba8()) == meta["rgba8_sha256"]


@pytest.mark.gpu
def test_gpu_mid_scene_full_size_matches_fixture_subset(ctx):
    """The full 8 x 2^18-ray mid scene traced on the GPU; the stored every-32749th-primary
    subset of the oracle's trace must be reproduced inside it."""
    segs, paths, s64 = load("mid_scene_subset")
    stride = INDEX["mid_scene_subset"]["stride"]
    pk = W.mid_scene().packed()
    pk.params.record_paths = 1
    ctx.upload(pk)
    st = ctx.trace()
    assert st["primary_rays"] == 8 << 18
    g_segs, g_paths = ctx.segments(paths=True)
    keep = (g_paths["source"] != abi.LG_SRC_TRACE) | (g_paths["primary"] % stride == 0)
    rep = compare(g_segs[keep], g_paths[keep], segs, paths, s64)
    assert rep.ok(), rep
    assert rep.matched > 0.99 * len(segs)


@pytest.mark.gpu
def test_gpu_default_scene_from_ron_matches_fixture(ctx):
    """The reference's shipped scene (default.ron, loaded through light_garden_gb300.ron):
    the GPU trace reproduces the stored oracle subset and the stored image digest."""
    from light_garden_gb300 import ron
    from light_garden_gb300.scene import pack
    meta = json.loads((GOLD / "default_scene.json").read_text())
    objs, lights = ron.load(GOLD / "default_scene.ron")
    p = abi.params_default()
    p.width, p.height = meta["width"], meta["height"]
    p.record_paths = 1
    pk = pack(objs, lights, p)
    ctx.upload(pk)
    ctx.trace()
    g_segs, g_paths = ctx.segments(paths=True)
    z = np.load(GOLD / "default_scene.npz")
    keep = (g_paths["source"] != abi.LG_SRC_TRACE) | (g_paths["primary"] % meta["stride"] == 0)
    rep = compare(g_segs[keep], g_paths[keep], z["segs"], z["paths"], z["s64"])
    assert rep.ok(), rep
    assert rep.matched > 0.99 * len(z["segs"])
    ctx.accumulate()
    assert ctx.accum().shape == (meta["height"], meta["width"], 4)


@pytest.mark.gpu
def test_gpu_nested_string_mod_matches_fixture(ctx):
    """A nested mod over the crossings of a hypotrochoid mod's lines: the GPU's lines equal
    the stored ones bit for bit, and its rendered frame has the stored image digests."""
    name = "nested_string_mod_hypotrochoid"
    meta = INDEX[name]
    ctx.upload(W.nested_string_mod_art(abi.LG_CURVE_HYPOTROCHOID).packed())
    img, st = ctx.render()
    assert ctx.chords().tobytes() == load_chords(name).tobytes()
    assert st["pixels"] == meta["pixels"]
    assert digest(ctx.accum()) == meta["accum_sha256"]
    assert digest(img) == meta["f16_sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in sorted(INDEX) if n.startswith("string_mod_")])
def test_gpu_string_mod_art_matches_fixture(ctx, name):
    """String-mod line art on each curve with modulo colours: the GPU's lines equal the stored
    ones bit for bit, and its rendered frame has the stored image digests."""
    curve = {"circle": abi.LG_CURVE_CIRCLE, "complex_exp": abi.LG_CURVE_COMPLEX_EXP,
             "hypotrochoid": abi.LG_CURVE_HYPOTROCHOID, "lissajous": abi.LG_CURVE_LISSAJOUS}[name[len("string_mod_"):]]
    meta = INDEX[name]
    ctx.upload(W.string_mod_art(curve).packed())
    img, st = ctx.render()
    assert ctx.chords().tobytes() == load_chords(name).tobytes()
    assert st["pixels"] == meta["pixels"]
    assert digest(ctx.accum()) == meta["accum_sha256"]
    assert digest(img) == meta["f16_sha256"]
