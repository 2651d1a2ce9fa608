"""The launch-shape autotuner's search and cache, on the CPU with a stand-in
for the GPU timing."""
import json

from eden_gb300 import autotune, lowering, workloads


def _low():
    return lowering.lower(workloads.multicomp_net(n_cells=20, in_degree=5, length_ms=2.0))


def test_window_bound_follows_min_delay():
    low = _low()
    assert autotune.window_bound(low) == min(31, int(low.syn_delay.min() // low.dt))
    izh = lowering.lower(workloads.izh_net(n_cells=50, in_degree=5, length_ms=2.0))
    assert autotune.candidates(izh)["segments_per_warp"] == [0]


def test_search_finds_the_minimum_of_each_knob():
    low = _low()
    best_of = {"segments_per_depth": 32, "segments_per_warp": 384, "steps_per_launch": 0}
    calls = []

    def fake(cfg):
        calls.append(cfg)
        return 1.0 + sum(0.1 for k, v in cfg.items() if v != best_of[k])

    best, tried = autotune.search(low, fake)
    assert {k: best[k] for k in autotune.KNOBS} == best_of
    assert abs(best["ms_per_step"] - 1.0) < 1e-12
    # each configuration is measured once
    assert len(calls) == len({tuple(c[k] for k in autotune.KNOBS) for c in calls}) == len(tried)


def test_result_is_cached_per_network_and_device(tmp_path):
    low = _low()
    path = str(tmp_path / "tune.json")
    n = [0]

    def fake(cfg):
        n[0] += 1
        return 2.0 - 0.5 * (cfg["segments_per_warp"] == 192)

    a = autotune.tune(low, cache=path, measure=fake, device_name="dev")
    assert not a["cached"] and a["segments_per_warp"] == 192 and n[0] > 1
    calls = n[0]
    b = autotune.tune(low, cache=path, measure=fake, device_name="dev")
    assert b["cached"] and n[0] == calls and autotune.options(b) == autotune.options(a)
    autotune.tune(low, cache=path, measure=fake, device_name="other")
    assert n[0] > calls
    assert len(json.load(open(path))) == 2
    other = lowering.lower(workloads.multicomp_net(n_cells=21, in_degree=5, length_ms=2.0))
    assert autotune.fingerprint(other, "dev") != autotune.fingerprint(low, "dev")
