"""Writes tests/golden/default_scene.ron and default_scene.npz from the reference's
shipped scene file.

    python tests/golden/make_ron_fixture.py path/to/default.ron

The reference ships one scene, ``default.ron`` (loaded by Tracer::load, tracer.rs:190-204).
This script parses it with light_garden_gb300.ron, writes it back in the same format
(``default_scene.ron``, so the tests do not need the reference checkout), and stores the
CPU oracle's trace of it (every 7th primary, canonical order) with image digests at
1024x768, for the GPU tests and the loader round trip.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from light_garden_gb300 import abi, ron  # noqa: E402
from light_garden_gb300.scene import pack  # noqa: E402
from oracle import oracle as O  # noqa: E402

STRIDE = 7
W, H = 1024, 768


def params():
    p = abi.params_default()
    p.width, p.height = W, H
    return p


def main():
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_ron_fixture.py path/to/default.ron (the reference checkout's scene file)")
    objects, lights = ron.load(Path(sys.argv[1]))
    text = ron.dumps(objects, lights)
    (HERE / "default_scene.ron").write_text(text)
    pk = pack(objects, lights, params())
    O.build()
    segs, paths, s64, st = O.trace(pk, ray_stride=STRIDE)
    order = np.lexsort((paths["path"], paths["gen"], paths["primary"], paths["light"], paths["source"]))
    np.savez_compressed(HERE / "default_scene.npz", segs=segs[order], paths=paths[order], s64=s64[order])
    fsegs, _, _, fst = O.trace(pk)
    acc, px = O.raster(fsegs, pk.params)
    meta = {"stride": STRIDE, "width": W, "height": H, "segments_subset": int(len(segs)),
            "segments": int(len(fsegs)), "pixels": px,
            "f16_sha256": hashlib.sha256(O.resolve_f16(acc).tobytes()).hexdigest()}
    (HERE / "default_scene.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
    print(meta)


if __name__ == "__main__":
    main()
