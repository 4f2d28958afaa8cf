"""Lookup of the autotuner's table (lowrankintegrators.jl_gb300/_tuning.py)
on the CPU: the ensemble entry follows the rank bucket holding most of a
batch's work, the stream entry the nearest snapshot shape, and missing
tables or entries give the built-in defaults.  Also checks that the
committed table, when present, has the fields the library reads."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
spec = importlib.util.spec_from_file_location("lri_tuning", os.path.join(ROOT, "lowrankintegrators.jl_gb300",
                                                                         "_tuning.py"))
T = importlib.util.module_from_spec(spec)
spec.loader.exec_module(T)

TABLE = {
    "ensemble": {"df": {"r23-64": {"ctas_per_sm": 2}, "r13-22": {"ctas_per_sm": 3}},
                 "fp32": {"r1-12": {"ctas_per_sm": 3}}},
    "stream": {"8192x4096x96": {"splits_rows": 2, "splits_cols": 4, "stages": 4},
               "1024x512x48": {"splits_rows": 4, "splits_cols": 6, "stages": 3}},
}


def test_rank_buckets():
    assert T.rank_bucket(4) == "r1-12" and T.rank_bucket(12) == "r1-12"
    assert T.rank_bucket(13) == "r13-22" and T.rank_bucket(23) == "r23-64" and T.rank_bucket(64) == "r23-64"


def test_ensemble_lookup_by_dominant_bucket():
    # three r = 32 instances outweigh ten r = 14 instances of the same size
    n = [500] * 13
    r = [14] * 10 + [32] * 3
    assert T.ensemble_occupancy("df", n, n, r, TABLE) == (2, "r23-64")
    assert T.ensemble_occupancy("df", n[:10], n[:10], r[:10], TABLE) == (3, "r13-22")
    assert T.ensemble_occupancy("fp32", [100], [100], [20], TABLE) == (3, None)  # no entry for the bucket
    assert T.ensemble_occupancy("df", [100], [100], [20], {}) == (3, None)


def test_stream_lookup_nearest_shape():
    assert T.stream_pass_tiles(8192, 4096, 96, TABLE) == (2, 4, 4, "8192x4096x96")
    assert T.stream_pass_tiles(6000, 4000, 80, TABLE)[3] == "8192x4096x96"
    assert T.stream_pass_tiles(1000, 600, 40, TABLE) == (4, 6, 3, "1024x512x48")
    assert T.stream_pass_tiles(1000, 600, 40, {}) == (0, 0, 0, None)


def test_committed_table_is_well_formed():
    table = T.load()
    if not table:
        return
    for prec, buckets in table.get("ensemble", {}).items():
        assert prec in ("fp32", "df")
        for b, e in buckets.items():
            assert e["ctas_per_sm"] in (2, 3)
    for key, e in table.get("stream", {}).items():
        assert len(key.split("x")) == 3
        assert e["splits_rows"] >= 0 and e["splits_cols"] >= 0 and e["stages"] in (0, 2, 3, 4)
