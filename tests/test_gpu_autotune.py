"""The launch-shape knobs and the autotuner on the GPU.  Forest packing
(compartments per warp and per depth) changes no compartment's operations
and no cell's elimination order, so the records are identical bit for bit;
a shorter window only changes the rounding of the synapses' closed-form
decay across window boundaries, so it is held to the parity tolerances."""
import numpy as np
import pytest

from criteria import box_violations, samecount
from eden_gb300 import autotune, lowering, workloads
from eden_gb300.engine import MODE_BATCHED, Simulation
from helpers import spike_trains

pytestmark = pytest.mark.gpu


def _net():
    return lowering.lower(workloads.multicomp_net(n_cells=40, in_degree=20, length_ms=20.0, max_seg=120,
                                                  n_recorded=8))


def _run(low, **kw):
    sim = Simulation(low, mode=MODE_BATCHED, **kw)
    try:
        return sim.run()
    finally:
        sim.close()


@pytest.mark.parametrize("spw,spd", [(192, 0), (0, 32), (100, 128), (1023, 16)])
def test_packing_does_not_change_results(spw, spd):
    low = _net()
    a = _run(low)
    b = _run(low, segments_per_warp=spw, segments_per_depth=spd)
    assert len(a.spike_src) > 0
    np.testing.assert_array_equal(a.trace, b.trace)
    np.testing.assert_array_equal(a.spike_src, b.spike_src)
    np.testing.assert_array_equal(a.spike_step, b.spike_step)


def test_shorter_windows_stay_within_parity_tolerance():
    low = _net()
    kmax = autotune.window_bound(low)
    a = _run(low)
    b = _run(low, steps_per_launch=max(1, kmax // 4))
    dt_ms = float(low.dt) * 1e-3
    wrong, far = samecount(spike_trains(a.spike_src, a.spike_step), spike_trains(b.spike_src, b.spike_step),
                           int(round(0.1 / dt_ms)))
    assert not wrong and not far
    nbad, worst = box_violations(a.trace, b.trace, dt_ms, 0.1, 0.5)
    assert nbad == 0, worst


def test_tune_returns_a_working_configuration(tmp_path):
    low = _net()
    res = autotune.tune(low, cache=str(tmp_path / "t.json"))
    assert not res["cached"] and res["ms_per_step"] > 0 and len(res["tried"]) >= 3
    assert res["ms_per_step"] <= min(t["ms_per_step"] for t in res["tried"]) + 1e-12
    rec = _run(low, **autotune.options(res))
    assert len(rec.spike_src) > 0
    again = autotune.tune(low, cache=str(tmp_path / "t.json"))
    assert again["cached"] and autotune.options(again) == autotune.options(res)
