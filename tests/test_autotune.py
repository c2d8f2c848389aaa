"""Host logic of the batched-kernel autotuner: the candidate table obeys the
C ABI's rules for launch shapes and variant flags, and the committed ranking's
best entry is what the runners load."""
import json

from mkfbodytracker_pdaf_gb300 import autotune

VEC, SEARCH, PAIR, LOWSMEM = 1, 2, 4, 8        # MKF_BPF_* in include/mkf_gb300.h


def _valid(tb, cps, var):
    if not (64 <= tb <= 512 and tb % 32 == 0 and 0 <= cps <= 32):
        return False
    if var & ~(VEC | SEARCH | PAIR | LOWSMEM):
        return False
    if var & LOWSMEM and ((var & (VEC | SEARCH)) != (VEC | SEARCH) or var & PAIR):
        return False
    return True


def test_candidates_are_valid_launch_choices():
    assert len(set(autotune.CANDIDATES)) == len(autotune.CANDIDATES)
    for c in autotune.CANDIDATES:
        assert _valid(*c), c
    assert set(autotune.QUICK) <= set(autotune.CANDIDATES)


def test_committed_ranking_and_load_tuning():
    with open(autotune.TUNING_FILE) as f:
        d = json.load(f)
    ok = [r for r in d["results"] if "ms" in r]
    best = min(ok, key=lambda r: r["ms"])
    assert d["best"] == best
    shape = autotune.load_tuning()
    assert shape == (best["block_threads"], best["ctas_per_sm"], best["variant"])
    assert _valid(*shape)
    assert shape in autotune.CANDIDATES


def test_quick_ranking_keeps_the_previous_table():
    old = {"when": "t0", "results": [{"block_threads": 256, "ctas_per_sm": 2, "variant": 0, "ms": 9.0}],
           "best": {"block_threads": 256, "ctas_per_sm": 2, "variant": 0, "ms": 9.0}}
    new = {"when": "t1", "results": [{"block_threads": 256, "ctas_per_sm": 3, "variant": 11, "ms": 5.0}],
           "best": {"block_threads": 256, "ctas_per_sm": 3, "variant": 11, "ms": 5.0}}
    m = autotune.merge_rankings(new, old)
    assert m["best"] == new["best"] and m["results"] == new["results"]
    assert m["earlier_results"] == {"when": "t0", "results": old["results"]}
    assert autotune.merge_rankings(new, None) is new
