"""Seven of the reference's own validation networks on the GPU, run by the
C++ host program (eden_gb300/host/eden_gpu_host) through the C ABI:
LEMS_EdenTest_CoreInputs (pulse, weighted pulse, sine, ramp and their DL
forms, voltage clamps, timed input, spike array and generator),
LEMS_EdenTest_PassiveCompartment, LEMS_EdenTest1 (three two-compartment
cells with frustum dendrites, a gap junction, an expOne connection, a
sodium gate's state recorded), LEMS_EdenTest2 (an HH cell with its m, h
and n recorded) and LEMS_EdenTest_DomainDecomposition (14 spiking
two-compartment cells, gap junctions, expOne connections; compared by the
reference's box(0.1 ms, 0.5 mV) criterion) and EdenTest_Extension_CustomSetup
(izhikevichCell instances and pulse inputs customised per instance, expOne
connections customised per connection, whose halves must be identical)
and LEMS_EdenTest_CoreSynapses (every core chemical and continuous
synapse, the blocking-plastic one with its block and plasticity; compared
by box(0.1 ms, 0.5 mV), as the reference checks this network against NEURON
with boxes of 10-50 us by 0.1-0.5 mV),
read by this package's NeuroML reader and lowered into
model files (tests/golden/make_validation_golden.py), against the
reference simulator's own output on the same files: every recorded
potential within the stated mV (0.01 for the networks without spikes; the
reference's kernels are compiled with -Ofast, and on a spike's upstroke V
moves 4-5 mV per step), every gate state within 1 % of that number."""
import os
import subprocess

import numpy as np
import pytest

from criteria import box_violations
from eden_gb300 import build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("mode", ["batched", "plain"])
@pytest.mark.parametrize("name,tol_mv", [("core_inputs", 0.01), ("passive_compartment", 0.01), ("edentest1", 0.05),
                                         ("edentest2", 0.05), ("domain_decomposition", None),
                                         ("custom_setup_ext", 0.1), ("core_synapses", None)])
def test_validation_network_on_gpu_matches_reference(name, tol_mv, mode, tmp_path):
    z = np.load(os.path.join(HERE, "golden", f"validation_{name}.npz"))
    traj, ev = str(tmp_path / "traj.txt"), str(tmp_path / "ev.txt")
    p = subprocess.run([build.build_host(), os.path.join(HERE, "golden", f"validation_{name}.egm"), traj, ev, mode],
                       capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    mine = np.loadtxt(traj, ndmin=2)[::int(z["stride"])]
    ref = np.column_stack([z["time_s"], z["values_si"]])
    assert mine.shape == ref.shape
    np.testing.assert_allclose(mine[:, 0], ref[:, 0], rtol=0, atol=1e-9)
    scale = z["scale"]  # SI per engine unit: 1e-3 for potentials, 1 for gate states
    if tol_mv is None:
        # spiking network: the reference's criterion, box(0.1 ms, 0.5 mV), on
        # the stored rows
        dt_ms = float(ref[1, 0] - ref[0, 0]) * 1e3
        nbad, worst = box_violations(ref[:, 1:] / scale, mine[:, 1:] / scale, dt_ms, 0.1, 0.5)
        assert nbad == 0, f"{nbad} samples outside box(0.1 ms, 0.5 mV), worst {worst} mV"
        return
    err = np.abs(mine[:, 1:] - ref[:, 1:]) / scale  # engine units
    tol = np.where(scale == 1.0, tol_mv * 1e-2, tol_mv)
    assert (err <= tol).all(), err.max(0)
    if name == "custom_setup_ext":
        # the reference's half_vs_half criteria
        # (testing/validation_tests/validation_tests.py:31-42): identical traces
        full = np.loadtxt(traj, ndmin=2)[:, 1:]
        for a, b in [(5, 0), (6, 1), (7, 2), (8, 3), (9, 4), (10, 12), (11, 13)]:
            np.testing.assert_array_equal(full[:, a], full[:, b])
