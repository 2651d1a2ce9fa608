"""Fixtures of the reference's own validation networks for the GPU.

Reads seven of the reference's validation networks
(testing/validation_tests/neuroml/LEMS_EdenTest_CoreInputs.xml,
LEMS_EdenTest_PassiveCompartment.xml, LEMS_EdenTest1.xml,
LEMS_EdenTest2.xml, LEMS_EdenTest_DomainDecomposition.xml,
LEMS_EdenTest_CoreSynapses.xml and
EdenTest_Extension_CustomSetup.nml with its custom setup file) with this
package's NeuroML reader,
writes each lowered network as a model file (eden_gb300/model_file.py) that
the C++ host program runs through the C ABI, and stores the reference
simulator's own trajectory output for the same file (oracle/_ref/eden,
built from the reference sources).  Needs the reference tree and its build.

    EDEN_REFERENCE_DIR=<reference tree> python tests/golden/make_validation_golden.py
"""
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import reference_runner  # noqa: E402
from eden_gb300 import lowering, model_file, neuroml_io  # noqa: E402

# fixture name -> (network file, the reference's trajectory output file or
# None for the one file it writes, trajectory rows kept: every stride-th)
NETWORKS = {
    "core_inputs": ("LEMS_EdenTest_CoreInputs.xml", "results.gen.txt", 1),
    "passive_compartment": ("LEMS_EdenTest_PassiveCompartment.xml", None, 16),
    "edentest1": ("LEMS_EdenTest1.xml", "results1.txt", 1),
    "edentest2": ("LEMS_EdenTest2.xml", "results1.txt", 1),
    "domain_decomposition": ("LEMS_EdenTest_DomainDecomposition.xml", "results.gen.txt", 4),
    "custom_setup_ext": ("EdenTest_Extension_CustomSetup.nml", "results.gen.txt", 4),
    "core_synapses": ("LEMS_EdenTest_CoreSynapses.xml", "results.gen.txt", 5),
}


def make(name):
    fname, outfile, stride = NETWORKS[name]
    path = reference_runner.validation_network(fname)
    if path is None:
        sys.exit("the reference tree is not present (set EDEN_REFERENCE_DIR)")
    spec = neuroml_io.read_lems(path)
    low = lowering.lower(spec)
    work = tempfile.mkdtemp(prefix="eden_val_")
    try:
        reference_runner.run(path, threads=2, keep_dir=work)
        files = [outfile] if outfile else [f for f in os.listdir(work) if f.endswith(".txt") and "spike" not in f
                                           and f not in os.listdir(os.path.dirname(path))]
        ref = np.loadtxt(os.path.join(work, files[0]), ndmin=2)
    finally:
        shutil.rmtree(work, ignore_errors=True)
    model_file.write_for_spec(os.path.join(HERE, f"validation_{name}.egm"), spec, low)
    ref = ref[::stride]
    # per column: SI value = engine value x scale (mV -> V; gate states as they are)
    scale = np.array([c[3] for of in spec.output_files for c in of["cols"]], np.float64)
    np.savez_compressed(os.path.join(HERE, f"validation_{name}.npz"), time_s=ref[:, 0], values_si=ref[:, 1:],
                        network=fname, stride=stride, scale=scale)
    print(f"{name}: {low.n_target} targets, {low.n_steps} steps, {ref.shape[1] - 1} columns")


if __name__ == "__main__":
    if not reference_runner.available():
        sys.exit("oracle/_ref/eden is not built (make -C oracle ref)")
    for n in sys.argv[1:] or list(NETWORKS):
        make(n)
