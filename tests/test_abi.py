"""The C ABI library: it builds for sm_103a, loads, exports every entry
point include/eden_gpu.h declares, and refuses to run without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from eden_gb300 import engine, lowering, workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "eden_gpu.h")).read()
    return sorted(set(re.findall(r"\b(edenGpu[A-Za-z]+)\s*\(", text)))


def test_header_matches_binding_list():
    assert declared_symbols() == sorted(engine.EXPORTED)


def test_library_exports_all_symbols():
    lib = engine.load_library()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.edenGpuAbiVersion() == lowering.ABI_VERSION


def test_struct_layouts_match_header():
    # sizes of the ctypes mirrors against offsets a C compiler computes
    assert ctypes.sizeof(lowering.CModel) % 8 == 0
    assert lowering.CHAN_DTYPE.itemsize == 4 + 10 * 4 * 4
    assert lowering.SYN_DTYPE.itemsize == 7 * 4


def test_create_without_gpu_fails_loudly():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is visible")
    except ImportError:
        pass
    low = lowering.lower(workloads.single_comp_hh(n_cells=4, length_ms=1.0))
    with pytest.raises(engine.EdenGpuError) as e:
        engine.Simulation(low)
    assert e.value.code == -6  # EDEN_GPU_E_NODEVICE
