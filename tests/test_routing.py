"""Synaptic event routing: the oracle's per-synapse results against an
independent restatement of the reference's delivery and single-pending-spike
rule (oracle/routing.py), given the same spike trains.  Bit-exact: the
pending slot of every synapse and the number of steps each synapse fired in.
The GPU side of the same check is in test_gpu_routing.py."""
import numpy as np
import pytest

import eden_port
import routing
from eden_gb300 import lowering
from golden.cases import spec_of


@pytest.mark.parametrize("name", ["izh_net", "multicomp_recurrent", "multicomp_poisson"])
def test_oracle_routing_matches_restatement(name):
    low = lowering.lower(spec_of(name))
    out = eden_port.run(low)
    assert out["rc"] == 0
    pend, fires = routing.route(low.syn_src, low.syn_delay, out["spike_src"], out["spike_step"], float(low.dt),
                                low.n_steps)
    assert np.array_equal(pend.view(np.uint32), out["syn_final_pending"].view(np.uint32))
    assert np.array_equal(fires, out["syn_fire_count"])
    assert fires.sum() > 0
    fast = routing.route_pending(low.syn_src, low.syn_delay, out["spike_src"], out["spike_step"], float(low.dt),
                                 low.n_steps)
    assert np.array_equal(fast.view(np.uint32), pend.view(np.uint32))


def test_single_pending_slot_drops_closely_spaced_spikes():
    # delay 1 ms, dt 0.1 ms: spikes read at steps 1, 3 and 12 -- the second
    # arrives while the first is still pending and is dropped
    pend, fires = routing.route([0], [1000.0], [0, 0, 0], [1, 3, 12], 100.0, 40)
    t = routing.step_times(100.0, 40)
    assert pend[0] == np.float32(t[12] + np.float32(1000.0))
    assert fires[0] == 2


# ---------------------------------------------------------------------------
# pinned to the reference's own per-synapse tables (tests/golden/routing_*.npz,
# read from the reference simulator's raw state dumps by
# tests/golden/make_routing_golden.py)
from golden.make_routing_golden import LENGTH_MS, VARIANTS  # noqa: E402
from golden_io import routing_fixture  # noqa: E402
from eden_gb300 import workloads  # noqa: E402


@pytest.mark.parametrize("variant", list(VARIANTS))
def test_routing_restatement_matches_reference_tables(variant):
    """oracle/routing.py replayed on the spike lists' emission steps gives the
    reference's pending slot after every step and its firing count, bit for
    bit: delays of whole and fractional steps, below one step, and spikes
    closer together than the delays."""
    low = lowering.lower(workloads.routing_probe(length_ms=LENGTH_MS, **VARIANTS[variant]))
    fx = routing_fixture(variant, len(low.syn_src))
    for last in (1, 2, 7, 40, 97, 150, 151, 233, fx.last_step):
        pend, fires = routing.route(low.syn_src, low.syn_delay, low.ext_src, low.ext_step, float(low.dt), last)
        want = fx.pending_after(last)
        bad = np.flatnonzero(pend.view(np.uint32) != want.view(np.uint32))
        assert len(bad) == 0, f"step {last}: {len(bad)} pending slots differ, e.g. {bad[:5]}"
        assert np.array_equal(fires, fx.fire_count_through(last)), f"step {last}: firing counts differ"
    assert fx.fire_count_through(fx.last_step).sum() > 1000


@pytest.mark.parametrize("variant", list(VARIANTS))
def test_oracle_routing_matches_reference_tables(variant):
    """The C restatement's final pending slots and firing counts equal the
    reference's on the same probe."""
    low = lowering.lower(workloads.routing_probe(length_ms=LENGTH_MS, **VARIANTS[variant]))
    fx = routing_fixture(variant, len(low.syn_src))
    out = eden_port.run(low, n_steps=fx.last_step)
    assert out["rc"] == 0
    assert np.array_equal(out["syn_final_pending"].view(np.uint32), fx.pending_after(fx.last_step).view(np.uint32))
    assert np.array_equal(out["syn_fire_count"], fx.fire_count_through(fx.last_step))


@pytest.mark.parametrize("variant", list(VARIANTS))
def test_firing_steps_match_reference_tables(variant):
    """Every synapse fires in the same steps as in the reference's tables
    (the steps its conductance jumps instead of decaying)."""
    low = lowering.lower(workloads.routing_probe(length_ms=LENGTH_MS, **VARIANTS[variant]))
    fx = routing_fixture(variant, len(low.syn_src))
    _, steps = routing.route_steps(low.syn_src, low.syn_delay, low.ext_src, low.ext_step, float(low.dt),
                                   fx.last_step)
    order = np.lexsort((fx.fire_step, fx.fire_syn))
    ref_syn, ref_step = fx.fire_syn[order], fx.fire_step[order]
    mine_syn = np.concatenate([np.full(len(x), s) for s, x in enumerate(steps)])
    mine_step = np.concatenate(steps)
    np.testing.assert_array_equal(mine_syn, ref_syn)
    np.testing.assert_array_equal(mine_step, ref_step)
