"""Writes the golden fixtures of ``tests/test_golden.py`` from the CPU oracle.

    python tests/golden/make_golden.py

The reference has no tests, no golden outputs and no buildable CPU path here (it is Rust and
its geometry crate is not on disk), so the fixtures are the FP64 oracle's own output on the
seeded workloads, pinned after the oracle passed the analytic known-answer tests of
``tests/test_oracle.py``.  They freeze the oracle against regressions and give the GPU
tests a stored answer that does not depend on rebuilding the oracle.

Each case stores the segments (x0, y0, x1, y1 f32 + RGBA f32), their path records and the
FP64 endpoints in canonical order (source, light, primary, generation, path bits), for every
``stride``-th primary ray of each light, the string-mod lines (two colours each), plus SHA-256
digests of the int64 image and the RGBA16F resolve where the full scene is traced.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from light_garden_gb300 import abi, workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

# name -> (workload factory, primary stride, whether the image digests are stored)
CASES = {
    "plain_small_fixed64": (lambda: W.plain_small(accum=abi.LG_ACCUM_FIXED64), 1, True),
    "mid_scene_subset": (lambda: W.mid_scene(), 8191, False),
    "csg_scene_subset": (lambda: W.csg_scene(), 65521, False),
}
for _curve, _name in ((abi.LG_CURVE_CIRCLE, "circle"), (abi.LG_CURVE_COMPLEX_EXP, "complex_exp"),
                      (abi.LG_CURVE_HYPOTROCHOID, "hypotrochoid"), (abi.LG_CURVE_LISSAJOUS, "lissajous")):
    CASES[f"string_mod_{_name}"] = ((lambda c=_curve: W.string_mod_art(c)), 1, True)
# a nested mod over the crossings of a hypotrochoid mod's lines (StringMod::nested)
CASES["nested_string_mod_hypotrochoid"] = ((lambda: W.nested_string_mod_art(abi.LG_CURVE_HYPOTROCHOID)), 1, True)


def canonical(segs, paths, s64):
    order = np.lexsort((paths["path"], paths["gen"], paths["primary"], paths["light"], paths["source"]))
    return segs[order], paths[order], s64[order]


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_case(name: str):
    make, stride, images = CASES[name]
    pk = make().packed()
    segs, paths, s64, st = O.trace(pk, ray_stride=stride, threads=0)
    segs, paths, s64 = canonical(segs, paths, s64)
    chords = O.string_mod_chords(pk.params)  # the sample starts at primary 0: the overlay is drawn
    meta = {"stride": stride, "segments": int(len(segs)), "primary_rays": int(st.primary_rays),
            "near_degenerate": int(st.near_degenerate), "width": pk.params.width, "height": pk.params.height,
            "chords": int(len(chords))}
    if images:
        acc, px = O.raster(segs, pk.params, threads=0, chords=chords)
        meta.update(pixels=px, accum_sha256=digest(acc), f16_sha256=digest(O.resolve_f16(acc)),
                    rgba8_sha256=digest(O.resolve_rgba8(acc)))
    return segs, paths, s64, chords, meta


def main(names=None):
    """Writes the fixtures of ``names`` (every case when none are given) and their entries in
    golden.json, keeping the other entries."""
    O.build()
    path = HERE / "golden.json"
    index = json.loads(path.read_text()) if names and path.exists() else {}
    for name in names or CASES:
        segs, paths, s64, chords, meta = run_case(name)
        np.savez_compressed(HERE / f"{name}.npz", segs=segs, paths=paths, s64=s64, chords=chords)
        index[name] = meta
        print(name, meta)
    path.write_text(json.dumps(index, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main(sys.argv[1:])
