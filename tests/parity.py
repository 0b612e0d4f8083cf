"""Path-keyed comparison of a GPU trace against the CPU oracle's trace.

Both sides key every segment by (source, light, primary, generation, path bits).

exact(): the bar of LG_PRECISION_EXACT.  The same segment set, and every segment's
endpoints, colour, hit object and TIR flag equal bit for bit; nothing is excused.  The
near-degenerate flag is reported, not compared: the oracle also raises it for decisions on
objects the GPU's FP32 search proved irrelevant.

compare(): the bar of LG_PRECISION_FAST (double-float).  Hit-object ids and the set of
segments match exactly outside the flagged set, and endpoints match within ENDPOINT_TOL
relative to max(1, |p|).  Flagged means LG_PATH_NEAR_DEGENERATE (a decision in the oracle's
1e-10 band, on either side) or LG_PATH_ILL_CONDITIONED (GPU side: the double-float ray's
rounding bound passed 1e-6, so chaotic amplification may have parted it from the FP64 path),
and includes every descendant of a flagged decision.  The report counts the pairs excused
only as ill-conditioned separately (`flagged_ill`).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

ENDPOINT_TOL = 1e-5
COLOR_TOL = 1e-6   # relative: a few f32 ulps from the f64 -> f32 rounding of the reflectance
NEAR = 1
ILL = 8  # LG_PATH_ILL_CONDITIONED


def _keys(paths: np.ndarray) -> np.ndarray:
    return (paths["source"].astype(np.uint64) << np.uint64(60)) ^ (paths["light"].astype(np.uint64) << np.uint64(44)) \
        ^ (paths["primary"].astype(np.uint64) << np.uint64(8)) ^ paths["gen"].astype(np.uint64)


@dataclass
class ParityReport:
    matched: int
    gpu_only: int
    oracle_only: int
    gpu_only_unflagged: int
    oracle_only_unflagged: int
    hit_mismatch_unflagged: int
    color_mismatch_unflagged: int
    max_endpoint_err: float
    flagged: int
    # the flagged pairs present on both sides, compared anyway (informative, not a bar)
    flagged_matched: int = 0
    flagged_hit_mismatch: int = 0
    flagged_max_endpoint_err: float = 0.0
    flagged_ill: int = 0  # pairs flagged only as ill-conditioned (no decision in a band)

    def ok(self) -> bool:
        return (self.gpu_only_unflagged == 0 and self.oracle_only_unflagged == 0 and
                self.hit_mismatch_unflagged == 0 and self.color_mismatch_unflagged == 0 and
                self.max_endpoint_err <= ENDPOINT_TOL)


def compare(g_segs, g_paths, o_segs, o_paths, o_s64, primary_filter=None) -> ParityReport:
    if primary_filter is not None:
        keep = (g_paths["source"] != 0) | primary_filter(g_paths["primary"])
        g_segs, g_paths = g_segs[keep], g_paths[keep]
    gi = {}
    for i, (k, p) in enumerate(zip(_keys(g_paths).tolist(), g_paths["path"].tolist())):
        gi[(k, p)] = i
    oi = {}
    for i, (k, p) in enumerate(zip(_keys(o_paths).tolist(), o_paths["path"].tolist())):
        oi[(k, p)] = i
    common = gi.keys() & oi.keys()
    g_only = gi.keys() - oi.keys()
    o_only = oi.keys() - gi.keys()
    gflag = (g_paths["flags"] & (NEAR | ILL)) != 0
    oflag = (o_paths["flags"] & (NEAR | ILL)) != 0
    g_band = (g_paths["flags"] & NEAR) != 0
    ig = np.array([gi[k] for k in common], dtype=np.int64)
    io = np.array([oi[k] for k in common], dtype=np.int64)
    flagged = gflag[ig] | oflag[io] if len(ig) else np.zeros(0, bool)
    clean_g, clean_o = ig[~flagged], io[~flagged]
    hit_mm = int((g_paths["hit"][clean_g] != o_paths["hit"][clean_o]).sum())
    gc = g_segs["color"][clean_g].astype(np.float64)
    oc = o_segs["color"][clean_o].astype(np.float64)
    col_mm = int((np.abs(gc - oc) > COLOR_TOL * np.maximum(np.abs(oc), 1e-30)).any(axis=1).sum())
    if len(clean_g):
        gp = np.stack([g_segs["x0"][clean_g], g_segs["y0"][clean_g], g_segs["x1"][clean_g], g_segs["y1"][clean_g]], 1)
        op = o_s64[clean_o]
        err = np.abs(gp.astype(np.float64) - op) / np.maximum(1.0, np.abs(op))
        max_err = float(err.max())
    else:
        max_err = 0.0
    fg, fo = ig[flagged], io[flagged]
    f_hit = int((g_paths["hit"][fg] != o_paths["hit"][fo]).sum())
    if len(fg):
        gpf = np.stack([g_segs["x0"][fg], g_segs["y0"][fg], g_segs["x1"][fg], g_segs["y1"][fg]], 1)
        f_err = float((np.abs(gpf.astype(np.float64) - o_s64[fo]) / np.maximum(1.0, np.abs(o_s64[fo]))).max())
    else:
        f_err = 0.0

    def excused(key, own_flag, other_index, other_flag):
        # flagged on its own side, or its parent is flagged on the other side (the trees
        # diverged below a near-degenerate decision)
        if own_flag:
            return True
        (k, path) = key
        gen = k & 0xff
        if gen == 0:
            return False
        parent = ((k & ~np.uint64(0xff).item()) | (gen - 1), path & ~(1 << (gen - 1)))
        j = other_index.get(parent)
        return j is not None and bool(other_flag[j])

    g_only_unf = sum(1 for k in g_only if not excused(k, gflag[gi[k]], oi, oflag))
    o_only_unf = sum(1 for k in o_only if not excused(k, oflag[oi[k]], gi, gflag))
    ill_only = int((flagged & ~g_band[ig] & ~((o_paths["flags"][io] & NEAR) != 0)).sum()) if len(ig) else 0
    return ParityReport(len(common), len(g_only), len(o_only), g_only_unf, o_only_unf, hit_mm, col_mm, max_err,
                        int(flagged.sum()) + len(g_only) + len(o_only) - g_only_unf - o_only_unf,
                        int(len(fg)), f_hit, f_err, ill_only)


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    d = np.linalg.norm((a - b).ravel())
    n = np.linalg.norm(b.ravel())
    return float(d / n) if n > 0 else float(d)


@dataclass
class ExactReport:
    segments: int
    gpu_only: int
    oracle_only: int
    endpoint_mismatch: int
    color_mismatch: int
    hit_mismatch: int
    tir_mismatch: int
    near_flag_differs: int  # informational

    def ok(self) -> bool:
        return (self.gpu_only == 0 and self.oracle_only == 0 and self.endpoint_mismatch == 0 and
                self.color_mismatch == 0 and self.hit_mismatch == 0 and self.tir_mismatch == 0)


def canonical(segs, paths):
    order = np.lexsort((paths["path"], paths["gen"], paths["primary"], paths["light"], paths["source"]))
    return segs[order], paths[order]


def exact(g_segs, g_paths, o_segs, o_paths) -> ExactReport:
    """Bit-for-bit comparison of two traces (any order on either side)."""
    gs, gp = canonical(g_segs, g_paths)
    os_, op = canonical(o_segs, o_paths)
    gk = list(zip(_keys(gp).tolist(), gp["path"].tolist()))
    ok = list(zip(_keys(op).tolist(), op["path"].tolist()))
    if gk != ok:  # align on the keys both have
        gi = {k: i for i, k in enumerate(gk)}
        oi = {k: i for i, k in enumerate(ok)}
        common = sorted(gi.keys() & oi.keys())
        g_only, o_only = len(gi) - len(common), len(oi) - len(common)
        ig = np.array([gi[k] for k in common], dtype=np.int64)
        io = np.array([oi[k] for k in common], dtype=np.int64)
        gs, gp, os_, op = gs[ig], gp[ig], os_[io], op[io]
    else:
        g_only = o_only = 0
    ge = np.stack([gs["x0"], gs["y0"], gs["x1"], gs["y1"]], 1).view(np.uint32)
    oe = np.stack([os_["x0"], os_["y0"], os_["x1"], os_["y1"]], 1).view(np.uint32)
    return ExactReport(
        segments=len(gs), gpu_only=g_only, oracle_only=o_only,
        endpoint_mismatch=int((ge != oe).any(axis=1).sum()),
        color_mismatch=int((gs["color"].view(np.uint32) != os_["color"].view(np.uint32)).any(axis=1).sum()),
        hit_mismatch=int((gp["hit"] != op["hit"]).sum()),
        tir_mismatch=int(((gp["flags"] ^ op["flags"]) & 2).astype(bool).sum()),
        near_flag_differs=int(((gp["flags"] ^ op["flags"]) & NEAR).astype(bool).sum()))
