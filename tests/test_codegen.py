"""Run-time code generation: the kernel sources the library embeds compile
with NVRTC for sm_103a together with a generated channel routine of the form
the library writes (eden_codegen.cuh), here on the host, without a GPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NVRTC = "/usr/local/cuda/lib64/libnvrtc.so.13"

PRELUDE = ("typedef signed char int8_t;\ntypedef unsigned char uint8_t;\ntypedef short int16_t;\n"
           "typedef unsigned short uint16_t;\ntypedef int int32_t;\ntypedef unsigned int uint32_t;\n"
           "typedef long long int64_t;\ntypedef unsigned long long uint64_t;\n"
           "typedef decltype(sizeof(0)) size_t;\n")

# the routine generated for one channel set: leak (no gates), then a
# channel with gates m^3 h, as channel_routines writes it
ROUTINE = """namespace eden {
#define EDEN_RTC_CHANNELS 1
__device__ __forceinline__ bool rtc_channels(int sig, const float *q, const float *CHG, const float *CHE,
                                             int c0, float v, float A, float &Ich, float &Gch) {
    switch (sig) {
    case 0: {
        { float fopen = 1.0f; const float gs = CHG[c0 + 0] * fopen;
          Ich += (gs * (CHE[c0 + 0] - v) * 1e-5f) * A; Gch += (gs * 1e-5f) * A; }
        { float fopen = 1.0f; fopen = fopen * q[0]; fopen = fopen * q[0]; fopen = fopen * q[0];
          fopen = fopen * q[1]; const float gs = CHG[c0 + 1] * fopen;
          Ich += (gs * (CHE[c0 + 1] - v) * 1e-5f) * A; Gch += (gs * 1e-5f) * A; }
        return true;
    }
    default: return false;
    }
}
}  // namespace eden
"""


def test_embedded_kernels_compile_with_nvrtc():
    if not os.path.exists(NVRTC):
        pytest.skip("NVRTC not installed")
    from eden_gb300 import build
    build.embed_rtc_sources()
    inc = open(os.path.join(ROOT, "eden_gb300", "csrc", "_rtc_src.inc")).read()
    parts = re.findall(r'R"EDENRTC\((.*?)\)EDENRTC"', inc, re.S)
    assert parts
    src = PRELUDE + ROUTINE + "".join(parts)
    lib = ctypes.CDLL(NVRTC)
    prog = ctypes.c_void_p()
    assert lib.nvrtcCreateProgram(ctypes.byref(prog), src.encode(), b"eden_rtc.cu", 0, None, None) == 0
    for name in (b"eden::k_inputs_t", b"eden::k_cells_t", b"eden::k_deliver_t"):
        assert lib.nvrtcAddNameExpression(prog, name) == 0
    opts = [b"--gpu-architecture=sm_103a", b"-std=c++17", b"-DEDEN_RTC=1"]
    rc = lib.nvrtcCompileProgram(prog, len(opts), (ctypes.c_char_p * len(opts))(*opts))
    size = ctypes.c_size_t()
    lib.nvrtcGetProgramLogSize(prog, ctypes.byref(size))
    log = ctypes.create_string_buffer(size.value)
    lib.nvrtcGetProgramLog(prog, log)
    assert rc == 0, log.value.decode()[-2000:]
    assert "error" not in log.value.decode()
    cubin = ctypes.c_size_t()
    lib.nvrtcGetCUBINSize(prog, ctypes.byref(cubin))
    assert cubin.value > 0
    for name in (b"eden::k_inputs_t", b"eden::k_cells_t", b"eden::k_deliver_t"):
        low = ctypes.c_char_p()
        assert lib.nvrtcGetLoweredName(prog, name, ctypes.byref(low)) == 0 and low.value
    lib.nvrtcDestroyProgram(ctypes.byref(prog))
