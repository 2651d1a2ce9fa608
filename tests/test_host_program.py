"""The C++ host program (eden_gb300/host/eden_gpu_host.cpp) and the lowered-
model file it reads (eden_gb300/model_file.py), without a GPU: the file
holds every EdenGpuModel field under its own name and reads back equal, and
the host, linked against the library, fills the struct, checks the ABI
version and stops with the library's message when no GPU is visible."""
import os
import subprocess

import numpy as np
import pytest

from eden_gb300 import build, lowering, model_file, neuroml_io
from eden_gb300.lowering import CModel
from golden.cases import spec_of


def test_model_file_round_trip(tmp_path):
    spec = spec_of("spike_sources")
    low = lowering.lower(spec)
    path = str(tmp_path / "m.egm")
    model_file.write(path, low)
    back = model_file.read(path)
    arrays = model_file.model_arrays(low)
    for name, _ in CModel._fields_:
        if name not in arrays:
            continue
        a = np.ascontiguousarray(arrays[name])
        if a.dtype.fields is not None:
            assert back[name].tobytes() == a.tobytes(), name
        else:
            np.testing.assert_array_equal(back[name], a, err_msg=name)
    assert int(back["n_src"][0]) == len(low.src_target)
    assert int(back["run.n_steps"][0]) == low.n_steps
    np.testing.assert_array_equal(back["run.trace_target"], low.trace_target)


@pytest.fixture(scope="module")
def host_bin():
    return build.build_host()


def test_host_without_gpu_stops_with_the_library_message(host_bin, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    lems = neuroml_io.write_lems(spec_of("single_comp_hh"), str(tmp_path))
    spec = neuroml_io.read_lems(lems)
    path = str(tmp_path / "m.egm")
    model_file.write_for_spec(path, spec, lowering.lower(spec))
    p = subprocess.run([host_bin, path, str(tmp_path / "t.txt"), str(tmp_path / "e.txt")], capture_output=True,
                       text=True)
    assert p.returncode == 1
    assert "GPU set-up failed" in p.stderr


def test_host_rejects_a_file_that_is_not_a_model(host_bin, tmp_path):
    bad = tmp_path / "x.egm"
    bad.write_bytes(b"not a model")
    p = subprocess.run([host_bin, str(bad), os.devnull, os.devnull], capture_output=True, text=True)
    assert p.returncode == 1 and "bad magic" in p.stderr
