"""Single precision against double: the oracle in float (the reference's
arithmetic) against the same loop in double (oracle/port, EDEN_PORT_DOUBLE)
on the golden networks.  The float results stay within the path's stated
error: equal spike counts, every spike within 0.1 ms, membrane potential
within 0.5 mV of the double-precision trajectory."""
import numpy as np
import pytest

import eden_port
from eden_gb300 import lowering
from golden.cases import CASES, spec_of
from helpers import compare_spikes


@pytest.mark.parametrize("name", list(CASES))
def test_float_oracle_within_stated_error_of_double(name):
    low = lowering.lower(spec_of(name))
    f32 = eden_port.run(low)
    f64 = eden_port.run(low, double=True)
    assert f32["rc"] == 0 and f64["rc"] == 0
    shift = int(round(0.1 / (float(low.dt) * 1e-3)))
    bad, worst = compare_spikes(f64["spike_src"], f64["spike_step"], f32["spike_src"], f32["spike_step"], shift)
    assert bad == 0 and worst <= shift
    if f32["trace"].size:
        assert np.abs(f32["trace"].astype(np.float64) - f64["trace"]).max() < 0.5
