"""Error behaviour through the C ABI: malformed models are refused at
creation with EDEN_GPU_E_INVALID and a message, misuse of a live context
returns an error code and leaves the context usable, and buffer overflows
are reported as EDEN_GPU_E_RANGE -- never a crash, exit or device fault."""
import numpy as np
import pytest

from eden_gb300 import lowering, workloads
from eden_gb300.engine import EdenGpuError, MODE_BATCHED, MODE_PLAIN, Simulation

pytestmark = pytest.mark.gpu

E_INVALID, E_RANGE = -1, -5


def _small():
    return lowering.lower(workloads.multicomp_net(n_cells=8, in_degree=5, length_ms=5.0, max_seg=20))


def test_parent_after_child_is_refused():
    low = _small()
    low.comp_parent = low.comp_parent.copy()
    a = low.phys_comp_off[1]
    low.comp_parent[a + 1] = 5   # a compartment whose parent comes after it
    with pytest.raises(EdenGpuError) as e:
        Simulation(low)
    assert e.value.code == E_INVALID and "parent" in str(e.value)


@pytest.mark.parametrize("bad", [-1.0, float("nan")])
def test_negative_or_nan_delay_is_refused(bad):
    low = _small()
    low.syn_delay = low.syn_delay.copy()
    low.syn_delay[3] = bad
    with pytest.raises(EdenGpuError) as e:
        Simulation(low)
    assert e.value.code == E_INVALID and "delay" in str(e.value)


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_BATCHED])
def test_misuse_leaves_the_context_usable(mode):
    low = _small()
    sim = Simulation(low, mode=mode, record_capacity_steps=16)
    try:
        sim.initialize()
        # steps must continue where the last call ended
        rc = sim.lib.edenGpuRun(sim.ctx, 5, 10)
        assert rc == E_INVALID
        # more steps than the trajectory buffer holds without a fetch
        rc = sim.lib.edenGpuRun(sim.ctx, 1, 40)
        assert rc == E_RANGE and "fetch" in sim._err()
        # a state read of the wrong length
        v = np.zeros(3, np.float32)
        assert sim.lib.edenGpuReadV(sim.ctx, v.ctypes.data, 3) == E_RANGE
        sim.run_steps(10)
        rec = sim.fetch()
        assert len(rec.trace_step) == 10 and np.isfinite(rec.trace).all()
    finally:
        sim.close()


def test_spike_log_overflow_is_reported():
    low = lowering.lower(workloads.izh_net(n_cells=300, in_degree=20, length_ms=50.0))
    sim = Simulation(low, spike_capacity=8)
    try:
        sim.initialize()
        with pytest.raises(EdenGpuError) as e:
            sim.run_steps(400)
            sim.fetch()
        assert e.value.code == E_RANGE and "spike" in str(e.value)
    finally:
        sim.close()


@pytest.mark.parametrize("fault", ["source_with_target", "unsorted", "early"])
def test_bad_spike_source_events_are_refused(fault):
    low = lowering.lower(workloads.spike_sources(length_ms=10.0))
    low.ext_src, low.ext_step = low.ext_src.copy(), low.ext_step.copy()
    if fault == "source_with_target":
        low.ext_src[0] = int(np.nonzero(low.src_target >= 0)[0][0])
    elif fault == "unsorted":
        low.ext_step[0] = low.ext_step[-1] + 5
    else:
        low.ext_step[0] = 1          # logged before any step has run
    with pytest.raises(EdenGpuError) as e:
        Simulation(low)
    assert e.value.code == E_INVALID and "spike-source event" in str(e.value)
