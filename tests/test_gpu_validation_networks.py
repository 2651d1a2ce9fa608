"""Two of the reference's own validation networks on the GPU, run by the C++
host program (eden_gb300/host/eden_gpu_host) through the C ABI:
LEMS_EdenTest_CoreInputs (pulse, weighted pulse, sine, ramp and their DL
forms, voltage clamps, timed input, spike array and generator) and
LEMS_EdenTest_PassiveCompartment, read by this package's NeuroML reader and
lowered into model files (tests/golden/make_validation_golden.py), against
the reference simulator's own output on the same files: every recorded
potential within 0.01 mV."""
import os
import subprocess

import numpy as np
import pytest

from eden_gb300 import build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("mode", ["batched", "plain"])
@pytest.mark.parametrize("name", ["core_inputs", "passive_compartment"])
def test_validation_network_on_gpu_matches_reference(name, mode, tmp_path):
    z = np.load(os.path.join(HERE, "golden", f"validation_{name}.npz"))
    traj, ev = str(tmp_path / "traj.txt"), str(tmp_path / "ev.txt")
    p = subprocess.run([build.build_host(), os.path.join(HERE, "golden", f"validation_{name}.egm"), traj, ev, mode],
                       capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    mine = np.loadtxt(traj, ndmin=2)[::int(z["stride"])]
    ref = np.column_stack([z["time_s"], z["values_si"]])
    assert mine.shape == ref.shape
    np.testing.assert_allclose(mine[:, 0], ref[:, 0], rtol=0, atol=1e-9)
    assert np.abs(mine[:, 1:] - ref[:, 1:]).max() * 1e3 < 0.01
