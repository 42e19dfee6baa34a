"""The committed autotuning tables: every entry is an admissible launch
geometry (CPU; the tuners themselves run in tests/test_gpu_batch.py)."""
import json
import os

from nr_gpu_ldpc_gb300 import autotune

MAX_THREADS = 384  # decode CTA size bound


def test_committed_tables_hold_admissible_points():
    files = [f for f in os.listdir(autotune.TUNING_DIR) if f.endswith(".json")]
    assert files
    for f in files:
        with open(os.path.join(autotune.TUNING_DIR, f)) as fh:
            d = json.load(fh)
        seen = set()
        for e in d["entries"]:
            bg, z, cpb = e["bg"], e["z"], e["cw_per_cta"]
            spt = e.get("sub_rows_per_thread", 1)
            assert bg in (1, 2) and (bg, z) not in seen
            seen.add((bg, z))
            assert spt in (1, 2) and z % spt == 0
            assert 1 <= cpb and cpb * (z // spt) <= MAX_THREADS, e
            if "tried" in e and "us_per_cw" in e:
                assert e["us_per_cw"] == min(t["us_per_cw"] for t in e["tried"])


def test_candidates_stay_below_the_largest_admissible():
    assert autotune.candidates(1) == [1]
    assert autotune.candidates(5) == [1, 2, 3, 4, 5]
    assert max(autotune.candidates(48)) == 48
