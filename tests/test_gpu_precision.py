"""The GPU path (single precision) against the double-precision oracle on
the golden networks, in both modes: equal spike counts and every spike
within 0.1 ms -- the spike-time error the batched path is measured at."""
import numpy as np
import pytest

import eden_port
from eden_gb300 import lowering
from eden_gb300.engine import MODE_BATCHED, MODE_PLAIN, Simulation
from golden.cases import CASES, spec_of
from helpers import compare_spikes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_BATCHED], ids=["plain", "batched"])
@pytest.mark.parametrize("name", list(CASES))
def test_gpu_within_stated_error_of_double(name, mode):
    low = lowering.lower(spec_of(name))
    f64 = eden_port.run(low, double=True)
    sim = Simulation(low, mode=mode)
    rec = sim.run()
    sim.close()
    shift = int(round(0.1 / (float(low.dt) * 1e-3)))
    bad, worst = compare_spikes(f64["spike_src"], f64["spike_step"], rec.spike_src, rec.spike_step, shift)
    assert bad == 0, f"{bad} cells with a different spike count"
    assert worst <= shift, f"a spike {worst} steps from the double-precision one"
