"""Accuracy of the GPU raytrace against the FP64 oracle, as numbers per configuration.

The bounds are those of the parity tests: hit/miss, entity id and return type agree on at least
99.999 % of the points, and every disagreement lies on a point the oracle flags as ambiguous (FP32
cannot resolve its FP64 answer within 1e-6 relative: edge, near miss, equal depths, range bound or a
tie in return selection); distances of points both sides hit (off the ambiguity band) agree within
1e-5 relative; non-hit distances are exact.

`evaluate` returns the record (agreement, ambiguous points, maximum, p99 and mean relative distance
error) and `record` prints it and, when RGL_ACCURACY_DIR names a directory, writes it there as
<name>.json so a run's figures can be collected.
"""
from __future__ import annotations

import json
import os

import numpy as np

MIN_AGREEMENT = 0.99999
MAX_REL_DISTANCE = 1e-5


class Tally:
    """Accumulates points of one configuration (several sensors or requests) before `finish`."""

    def __init__(self):
        self.points = 0
        self.mism = 0
        self.mism_outside = 0
        self.amb = 0
        self.hits = 0
        self.nonhit_exact = True
        self.return_type_exact = True
        self.rel = []
        self.examples = []

    def add(self, rgl, got, exp, tag=None):
        amb = exp["ambiguous"] != 0
        hit_g, hit_e = got[rgl.RGL_FIELD_IS_HIT_I32], exp["is_hit"]
        ent_g, ent_e = got[rgl.RGL_FIELD_ENTITY_ID_I32], exp["entity_id"]
        mism = (hit_g != hit_e) | (ent_g != ent_e)
        rt = got.get(rgl.RGL_FIELD_RETURN_TYPE_U8)
        if rt is not None:
            self.return_type_exact &= bool(np.array_equal(rt, exp["return_type"]))
        both = (hit_g == 1) & (hit_e == 1) & ~amb
        dg, de = got[rgl.RGL_FIELD_DISTANCE_F32][both], exp["distance"][both]
        rel = np.abs(dg.astype(np.float64) - de.astype(np.float64)) / np.maximum(np.abs(de.astype(np.float64)), 1e-6)
        nh = (hit_g == 0) & (hit_e == 0)
        self.nonhit_exact &= bool(np.array_equal(got[rgl.RGL_FIELD_DISTANCE_F32][nh], exp["distance"][nh]))
        self.points += int(hit_g.size)
        self.mism += int(mism.sum())
        self.mism_outside += int((mism & ~amb).sum())
        for i in np.nonzero(mism & ~amb)[0][: max(0, 10 - len(self.examples))]:
            self.examples.append({"tag": tag, "point": int(i), "gpu": [int(hit_g[i]), int(ent_g[i]), float(got[rgl.RGL_FIELD_DISTANCE_F32][i])],
                                  "oracle": [int(hit_e[i]), int(ent_e[i]), float(exp["distance"][i])]})
        self.amb += int(amb.sum())
        self.hits += int(both.sum())
        self.rel.append(rel)
        return rel

    def finish(self, **extra):
        rel = np.concatenate(self.rel) if self.rel else np.zeros(0)
        out = {
            "points": self.points,
            "agreement_pct": 100.0 * (1.0 - self.mism / max(self.points, 1)),
            "mismatched_points": self.mism,
            "mismatches_outside_ambiguity_band": self.mism_outside,
            "ambiguous_points": self.amb,
            "hit_points_compared": self.hits,
            "max_rel_distance_error": float(rel.max(initial=0.0)),
            "p99_rel_distance_error": float(np.quantile(rel, 0.99)) if rel.size else 0.0,
            "mean_rel_distance_error": float(rel.mean()) if rel.size else 0.0,
            "nonhit_distances_exact": self.nonhit_exact,
            "return_types_exact": self.return_type_exact,
        }
        if self.examples:
            out["mismatch_examples"] = self.examples
        out.update(extra)
        return out


def evaluate(rgl, got, exp, **extra):
    t = Tally()
    rel = t.add(rgl, got, exp)
    return t.finish(**extra), rel


def assert_within_bounds(stats, min_agreement=MIN_AGREEMENT):
    assert stats["mismatches_outside_ambiguity_band"] == 0, \
        f"{stats['mismatches_outside_ambiguity_band']} non-ambiguous mismatches, e.g. {stats.get('mismatch_examples')}"
    assert stats["agreement_pct"] >= 100.0 * min_agreement, f"agreement {stats['agreement_pct']} %"
    assert stats["max_rel_distance_error"] <= MAX_REL_DISTANCE, f"max rel distance error {stats['max_rel_distance_error']}"
    assert stats["nonhit_distances_exact"], "non-hit distances differ"
    assert stats["return_types_exact"], "return types differ"


def record(name: str, stats: dict) -> None:
    line = json.dumps({"config": name, **stats}, sort_keys=True)
    print(line)
    d = os.environ.get("RGL_ACCURACY_DIR")
    if d:
        os.makedirs(d, exist_ok=True)
        with open(os.path.join(d, name + ".json"), "w") as f:
            f.write(line + "\n")
