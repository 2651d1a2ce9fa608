"""Synaptic event routing on the GPU, bit-exact: given the spike trains the
GPU produced, every synapse's pending-spike slot must equal the reference's
delivery and single-pending-spike rule replayed on the CPU
(oracle/routing.py), at several points of the run and in both execution
modes.  A one-step run before each check makes the batched path apply the
last window's triggers (it replays them at the start of the next window)."""
import numpy as np
import pytest

import routing
from eden_gb300 import lowering
from eden_gb300.engine import MODE_BATCHED, MODE_PLAIN, Simulation
from golden.cases import spec_of

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_BATCHED])
@pytest.mark.parametrize("name", ["izh_net", "multicomp_recurrent", "multicomp_poisson"])
def test_pending_slots_bit_exact(name, mode):
    low = lowering.lower(spec_of(name))
    sim = Simulation(low, mode=mode)
    try:
        sim.initialize()
        src, step = [], []
        checked = 0
        for chunk in (237, 1, 150, 1, 0):
            if chunk == 0 or sim.next_step > low.n_steps:
                break
            sim.run_steps(min(chunk, low.n_steps + 1 - sim.next_step))
            rec = sim.fetch()
            src.append(rec.spike_src)
            step.append(rec.spike_step)
            if chunk != 1:
                continue
            last = sim.next_step - 1
            s, k = np.concatenate(src), np.concatenate(step)
            want, _ = routing.route(low.syn_src, low.syn_delay, s, k, float(low.dt), last)
            got, _, _ = sim.read_synapses()
            bad = np.flatnonzero(got.view(np.uint32) != want.view(np.uint32))
            assert len(bad) == 0, f"step {last}: {len(bad)} synapses differ, e.g. {bad[:5]}"
            assert np.isfinite(want).any()
            checked += 1
        assert checked == 2
    finally:
        sim.close()


from golden.make_routing_golden import LENGTH_MS, VARIANTS  # noqa: E402
from golden_io import routing_fixture  # noqa: E402
from eden_gb300 import workloads  # noqa: E402


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_BATCHED], ids=["plain", "batched"])
@pytest.mark.parametrize("variant", list(VARIANTS))
def test_pending_slots_equal_reference_tables(variant, mode):
    """The GPU's pending slot of every synapse equals the reference
    simulator's own table (tests/golden/routing_*.npz) bit for bit, at
    points spread over the run: one-step windows, five-step windows replayed
    at the next window, and delays below one step."""
    low = lowering.lower(workloads.routing_probe(length_ms=LENGTH_MS, **VARIANTS[variant]))
    fx = routing_fixture(variant, len(low.syn_src))
    sim = Simulation(low, mode=mode)
    try:
        sim.initialize()
        checked = 0
        for chunk in (6, 1, 33, 1, 57, 1, 99, 1, 0):
            if chunk == 0:
                break
            sim.run_steps(chunk)
            sim.fetch()
            if chunk != 1:
                continue
            last = sim.next_step - 1
            got, _, _ = sim.read_synapses()
            want = fx.pending_after(last)
            bad = np.flatnonzero(got.view(np.uint32) != want.view(np.uint32))
            assert len(bad) == 0, f"step {last}: {len(bad)} synapses differ from the reference, e.g. {bad[:5]}"
            checked += 1
        assert checked == 4
    finally:
        sim.close()
