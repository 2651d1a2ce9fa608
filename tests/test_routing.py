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
