"""The bench-size networks on the GPU, checked through properties that hold
at any size, where the oracle would take too long:

* routing: every synapse's pending-spike slot equals the reference's
  delivery and single-pending-spike rule replayed from the GPU's own spike
  log (oracle/routing.py), bit for bit;
* parity at full size over the first 400 steps (10 ms) of multicomp_net
  against the oracle: the parity tests' samecount(0.1 ms) and
  box(0.1 ms, 0.5 mV), in both modes;
* bounds: every membrane potential finite (inside [-100, +70] mV for the
  cable cells; an izhikevich v may overshoot vpeak by one step before its
  reset), every spike logged at most once per cell and step.

multicomp_net: 10,000 cells, 797,757 compartments, 1 M expTwo synapses and
1 M Poisson inputs (dt 0.025 ms, 10 ms).  izh_net: 100,000 izhikevich cells,
10 M expOne synapses (dt 0.1 ms, 20 ms).  mixed_scale: 160,000 izhikevich
cells and 40,000 100-compartment trees (4.16 M compartments), 20 M expTwo
synapses and 20 M Poisson inputs (dt 0.025 ms, 5 ms)."""
import numpy as np
import pytest

import eden_port
import routing
from criteria import box_violations, samecount
from helpers import spike_trains
from eden_gb300 import lowering, workloads
from eden_gb300.engine import MODE_BATCHED, MODE_PLAIN, Simulation

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,length_ms", [("multicomp_net", 10.0), ("izh_net", 20.0), ("mixed_scale", 5.0)])
def test_full_size_routing_and_bounds(name, length_ms):
    low = lowering.lower(workloads.CONFIGS[name](length_ms=length_ms))
    sim = Simulation(low, mode=MODE_BATCHED, record_capacity_steps=low.n_steps + 8, spike_capacity=1 << 24)
    try:
        sim.initialize()
        sim.run_steps(low.n_steps)
        sim.run_steps(1)  # applies the last window's triggers
        rec = sim.fetch()
        last = sim.next_step - 1
        assert len(rec.spike_src) > 0
        pairs = rec.spike_src.astype(np.int64) * (last + 2) + rec.spike_step
        assert len(np.unique(pairs)) == len(pairs)
        want = routing.route_pending(low.syn_src, low.syn_delay, rec.spike_src, rec.spike_step, float(low.dt), last)
        got, _, _ = sim.read_synapses()
        bad = np.flatnonzero(got.view(np.uint32) != want.view(np.uint32))
        assert len(bad) == 0, f"{len(bad)} of {len(got)} pending slots differ, e.g. {bad[:5]}"
        v = sim.read_v()
        assert np.isfinite(v).all()
        if low.n_comp:
            cable = v[:low.n_comp]
            assert cable.min() > -100.0 and cable.max() < 70.0
        assert np.isfinite(rec.trace).all()
    finally:
        sim.close()


@pytest.fixture(scope="module")
def full_multicomp():
    low = lowering.lower(workloads.multicomp_net(length_ms=10.0))
    return low, eden_port.run(low, n_steps=400)


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_BATCHED], ids=["plain", "batched"])
def test_full_size_parity_first_10ms(full_multicomp, mode):
    low, ref = full_multicomp
    sim = Simulation(low, mode=mode, record_capacity_steps=408)
    try:
        rec = sim.run(400)
    finally:
        sim.close()
    shift = int(round(0.1 / (float(low.dt) * 1e-3)))
    wrong, far = samecount(spike_trains(ref["spike_src"], ref["spike_step"]),
                           spike_trains(rec.spike_src, rec.spike_step), shift)
    assert not wrong, f"{len(wrong)} cells with a different spike count, e.g. {wrong[:5]}"
    assert not far, f"{len(far)} cells with a spike more than 0.1 ms off, e.g. {far[:5]}"
    nbad, worst = box_violations(ref["trace"], rec.trace, float(low.dt) * 1e-3, 0.1, 0.5)
    assert nbad == 0, f"{nbad} samples outside box(0.1 ms, 0.5 mV), worst {worst} mV"
