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
    return sorted(set(re.findall(r"\b(edenGpu[A-Za-z0-9]+)\s*\(", text)))


def test_header_matches_binding_list():
    assert declared_symbols() == sorted(engine.EXPORTED)


def test_library_exports_all_symbols():
    lib = engine.load_library()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.edenGpuAbiVersion() == lowering.ABI_VERSION


def _c_layout(tmp_path, struct, fields):
    """sizeof(struct) and offsetof(struct, f) for each field, as the C
    compiler lays out include/eden_gpu.h."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "probe.c"
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "eden_gpu.h"', "int main(void) {",
             f'  printf("%zu\\n", sizeof({struct}));']
    lines += [f'  printf("%zu\\n", offsetof({struct}, {f}));' for f in fields]
    lines += ["  return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "probe"
    subprocess.run([cc, "-I", os.path.join(root, "include"), str(src), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    return out[0], out[1:]


def test_struct_layouts_match_header(tmp_path):
    # the ctypes / numpy mirrors against the offsets a C compiler computes
    for dtype, struct in ((lowering.CHAN_DTYPE, "EdenGpuChannelType"), (lowering.SYN_DTYPE, "EdenGpuSynapseType")):
        size, offs = _c_layout(tmp_path, struct, dtype.names)
        assert dtype.itemsize == size, struct
        assert [dtype.fields[f][1] for f in dtype.names] == offs, struct
    names = [f[0] for f in lowering.CModel._fields_]
    size, offs = _c_layout(tmp_path, "EdenGpuModel", names)
    assert ctypes.sizeof(lowering.CModel) == size
    assert [getattr(lowering.CModel, f).offset for f in names] == offs


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
