"""Tuned tile choices (``tuning.json``, written by ``autotune.py`` on the
target GPU) and their lookup.

Two tables:

``ensemble``  register budget of the instance engine's step kernel
              (``lri_batch_set_occupancy``: 3 or 2 CTAs per SM) per
              precision class and rank bucket; a batch takes the choice of
              the bucket that holds most of its work ((n + m) r^2 summed).
``stream``    K splits per 128-row tile of the tensor-core snapshot passes
              (dY X and dY^T X) and their pipeline stages, per snapshot
              shape; a stream takes the entry of the nearest shape (log
              distance in n, m, r_max).

Missing entries mean the built-in defaults (3 CTAs per SM; splits that fill
the SMs and as many stages as fit).
"""
from __future__ import annotations

import json
import math
import os
from typing import Dict, Optional, Sequence, Tuple

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE_PATH = os.path.join(HERE, "tuning.json")

# rank buckets of the ensemble table (inclusive upper bounds)
RANK_BUCKETS = (12, 22, 64)


def load(path: Optional[str] = None) -> Dict:
    p = path or TABLE_PATH
    if not os.path.exists(p):
        return {}
    with open(p) as f:
        return json.load(f)


def rank_bucket(r: int) -> str:
    lo = 1
    for hi in RANK_BUCKETS:
        if r <= hi:
            return f"r{lo}-{hi}"
        lo = hi + 1
    return f"r{lo}+"


def ensemble_occupancy(precision: str, n: Sequence[int], m: Sequence[int], r: Sequence[int],
                       table: Optional[Dict] = None) -> Tuple[int, Optional[str]]:
    """(CTAs per SM, bucket used) for a batch of the given precision and
    shapes; (3, None) without a tuned entry."""
    t = (load() if table is None else table).get("ensemble", {}).get(precision, {})
    if not t:
        return 3, None
    work: Dict[str, float] = {}
    for ni, mi, ri in zip(n, m, r):
        b = rank_bucket(int(ri))
        work[b] = work.get(b, 0.0) + float(ni + mi) * float(ri) ** 2
    best = max(work, key=work.get)
    e = t.get(best)
    if not e:
        return 3, None
    return int(e["ctas_per_sm"]), best


def stream_pass_tiles(n: int, m: int, R: int, table: Optional[Dict] = None
                      ) -> Tuple[int, int, int, Optional[str]]:
    """(splits_rows, splits_cols, stages, shape key used); zeros (automatic)
    without a tuned entry."""
    t = (load() if table is None else table).get("stream", {})
    if not t:
        return 0, 0, 0, None

    def dist(key):
        kn, km, kr = (int(x) for x in key.split("x"))
        return (math.log(n / kn) ** 2 + math.log(m / km) ** 2 + math.log(R / kr) ** 2)

    key = min(t, key=dist)
    e = t[key]
    return int(e["splits_rows"]), int(e["splits_cols"]), int(e["stages"]), key
