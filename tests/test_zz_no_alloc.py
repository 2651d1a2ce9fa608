"""edenGpuRunStaticScratch -- the step loop with its input scratch and window
table in static device arrays, allocating nothing -- against edenGpuRun on
the same model, through the C ABI.

Two contexts are built from one lowered model; one advances with edenGpuRun,
the other with edenGpuRunStaticScratch, over the same two calls in a row.
The same kernels run in the same order on the same inputs, so the records
are identical bit for bit (TRACE_ATOL_MV = 0); and after the one-time
set-up the device's free memory is the same before and after each call.
This file sorts last so that it also runs after every other GPU test in one
process."""
import ctypes

import numpy as np
import pytest
import torch

from eden_gb300 import engine, lowering, workloads
from golden.cases import spec_of

pytestmark = pytest.mark.gpu

TRACE_ATOL_MV = 0.0


def _free_bytes():
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info(0)[0]


def _static_entry(sim):
    f = sim.lib.edenGpuRunStaticScratch
    f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64]
    f.restype = ctypes.c_int
    return f


def _run_static(sim, n_steps):
    rc = _static_entry(sim)(sim.ctx, ctypes.c_int64(sim.next_step), ctypes.c_int64(n_steps))
    if rc != 0:
        raise engine.EdenGpuError(rc, sim._err())
    sim.next_step += n_steps


def _same_records(a, b):
    np.testing.assert_array_equal(a.trace_step, b.trace_step)
    np.testing.assert_allclose(b.trace, a.trace, rtol=0, atol=TRACE_ATOL_MV)
    np.testing.assert_array_equal(a.spike_src, b.spike_src)
    np.testing.assert_array_equal(a.spike_step, b.spike_step)


@pytest.mark.parametrize("mode", [engine.MODE_BATCHED, engine.MODE_PLAIN])
@pytest.mark.parametrize("case", ["izh_net", "multicomp_recurrent", "multicomp_poisson"])
def test_static_scratch_matches_run(case, mode):
    low = lowering.lower(spec_of(case))
    ref = engine.Simulation(low, mode=mode)
    sim = engine.Simulation(low, mode=mode)
    try:
        _run_static(sim, 0)            # one-time set-up only
        assert sim.next_step == -3
        ref.initialize()
        _run_static(sim, 4)            # the four initialisation passes
        half = low.n_steps // 2
        spikes = 0
        for n in (half, low.n_steps - half):   # two calls in a row
            ref.run_steps(n)
            free0 = _free_bytes()
            _run_static(sim, n)
            assert _free_bytes() == free0, "edenGpuRunStaticScratch changed the device's free memory"
            a, b = ref.fetch(), sim.fetch()
            assert len(a.trace_step) == n
            _same_records(a, b)
            spikes += len(a.spike_src)
        assert spikes > 0
        np.testing.assert_allclose(sim.read_v(), ref.read_v(), rtol=0, atol=TRACE_ATOL_MV)
    finally:
        ref.close()
        sim.close()


def test_static_scratch_interleaves_with_run():
    low = lowering.lower(spec_of("izh_net"))
    ref = engine.Simulation(low)
    sim = engine.Simulation(low)
    try:
        ref.initialize()
        sim.initialize()
        ref.run_steps(1000)
        sim.run_steps(300)
        _run_static(sim, 400)
        sim.run_steps(300)
        _same_records(ref.fetch(), sim.fetch())
    finally:
        ref.close()
        sim.close()


def test_static_scratch_rejects_models_beyond_its_size():
    # 80000 point neurons, each with a pulse and excitatory and inhibitory
    # synapses: about 231000 input chunks, more than the 131072 the static
    # scratch holds
    low = lowering.lower(workloads.izh_net(n_cells=80000, in_degree=10, length_ms=1.0, n_recorded=1))
    sim = engine.Simulation(low)
    try:
        with pytest.raises(engine.EdenGpuError) as e:
            _run_static(sim, 4)
        assert e.value.code == -5  # EDEN_GPU_E_RANGE
        assert "static scratch holds 131072" in str(e.value)
        assert sim.next_step == -3
        sim.initialize()           # the context is still usable through edenGpuRun
        sim.run_steps(8)
    finally:
        sim.close()
