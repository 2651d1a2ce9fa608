"""Python binding of libeden_gpu (include/eden_gpu.h) and the simulation driver.

`Simulation` owns one device context: it uploads a `LoweredModel`, advances
it through `edenGpuRun`, and collects the trajectory samples and spike
events the reference's loggers would write (eden/Eden.cpp:11555-11635).

There is no CPU fallback: if the compiled library cannot be loaded, or no
GPU is visible, construction raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build
from .lowering import LoweredModel, to_cmodel

MODE_PLAIN = 0
MODE_BATCHED = 1

_lib = None


class EdenGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"libeden_gpu error {code}: {msg}")
        self.code = code


class COptions(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("device", ctypes.c_int32),
                ("steps_per_launch", ctypes.c_int32), ("cells_per_block", ctypes.c_int32),
                ("record_capacity_steps", ctypes.c_int32), ("spike_capacity", ctypes.c_int32),
                ("n_trace", ctypes.c_int32), ("trace_target", ctypes.POINTER(ctypes.c_int32)),
                ("kernel_timing", ctypes.c_int32), ("codegen", ctypes.c_int32),
                ("max_cell_blocks", ctypes.c_int32), ("segments_per_warp", ctypes.c_int32),
                ("segments_per_depth", ctypes.c_int32), ("reserved", ctypes.c_int32 * 3)]


class CRecords(ctypes.Structure):
    _fields_ = [("trace", ctypes.POINTER(ctypes.c_float)), ("trace_step", ctypes.POINTER(ctypes.c_int64)),
                ("trace_capacity", ctypes.c_int64), ("spike_src", ctypes.POINTER(ctypes.c_int32)),
                ("spike_step", ctypes.POINTER(ctypes.c_int64)), ("spike_capacity", ctypes.c_int64),
                ("n_trace_samples", ctypes.c_int64), ("n_spikes", ctypes.c_int64),
                ("spike_time_us", ctypes.POINTER(ctypes.c_double))]


EXPORTED = ["edenGpuCreate", "edenGpuRun", "edenGpuRunStaticScratch", "edenGpuFetchRecords", "edenGpuGeneratedSource", "edenGpuReadV", "edenGpuWriteV", "edenGpuFp64Cells",
            "edenGpuReadSynapses", "edenGpuLastRunStats", "edenGpuKernelStats", "edenGpuLastError",
            "edenGpuDestroy", "edenGpuAbiVersion", "edenGpuGradCreate", "edenGpuGradForward",
            "edenGpuGradBackward", "edenGpuGradTiming", "edenGpuGradLastError", "edenGpuGradDestroy"]
KERNEL_NAMES = ["k_inputs_t", "k_cells_t", "k_targets_t", "k_hines_t", "k_deliver_t"]


def load_library(path: str | None = None, build_if_missing: bool = True):
    """Load libeden_gpu.so (building it in-tree first if needed)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    lib_path = path or _build.LIB
    if build_if_missing and path is None and _build.needs_build():
        _build.build()
    if not os.path.exists(lib_path):
        raise RuntimeError(f"libeden_gpu.so not found at {lib_path}; run eden_gb300/build.py")
    lib = ctypes.CDLL(lib_path)
    P = ctypes.c_void_p
    lib.edenGpuCreate.argtypes = [P, P, ctypes.POINTER(P)]
    lib.edenGpuCreate.restype = ctypes.c_int
    lib.edenGpuRun.argtypes = [P, ctypes.c_int64, ctypes.c_int64]
    lib.edenGpuRun.restype = ctypes.c_int
    lib.edenGpuFetchRecords.argtypes = [P, P]
    lib.edenGpuFetchRecords.restype = ctypes.c_int
    lib.edenGpuReadV.argtypes = [P, P, ctypes.c_int64]
    lib.edenGpuReadV.restype = ctypes.c_int
    lib.edenGpuWriteV.argtypes = [P, P, ctypes.c_int64]
    lib.edenGpuWriteV.restype = ctypes.c_int
    lib.edenGpuReadSynapses.argtypes = [P, P, P, P, ctypes.c_int64]
    lib.edenGpuReadSynapses.restype = ctypes.c_int
    lib.edenGpuLastRunStats.argtypes = [P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)]
    lib.edenGpuLastRunStats.restype = ctypes.c_int
    lib.edenGpuKernelStats.argtypes = [P, ctypes.c_int32, ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_int64)]
    lib.edenGpuKernelStats.restype = ctypes.c_int
    lib.edenGpuGeneratedSource.argtypes = [P, ctypes.c_char_p, ctypes.c_int64]
    lib.edenGpuGeneratedSource.restype = ctypes.c_int64
    lib.edenGpuLastError.argtypes = [P]
    lib.edenGpuLastError.restype = ctypes.c_char_p
    lib.edenGpuDestroy.argtypes = [P]
    lib.edenGpuDestroy.restype = None
    lib.edenGpuAbiVersion.argtypes = []
    lib.edenGpuAbiVersion.restype = ctypes.c_int
    if path is None:
        _lib = lib
    return lib


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


@dataclass
class Records:
    trace: np.ndarray        # [n_samples, n_trace] float32, mV
    trace_step: np.ndarray   # [n_samples] step index of each sample
    spike_src: np.ndarray    # [n_spikes] spike source (gid)
    spike_step: np.ndarray   # [n_spikes] logging step (the step after the crossing)
    spike_time: np.ndarray | None = None  # [n_spikes] crossing time in us interpolated in double (NaN: none)


class Simulation:
    """A lowered network on one GPU.

    mode: MODE_PLAIN (one set of launches per step) or MODE_BATCHED
    (windows of `steps_per_launch` steps, graph-replayed).
    """

    def __init__(self, lowered: LoweredModel, mode: int = MODE_BATCHED, device: int = 0,
                 steps_per_launch: int = 0, cells_per_block: int = 0, trace_target=None,
                 record_capacity_steps: int = 4096, spike_capacity: int = 1 << 22,
                 kernel_timing: bool = False, codegen: int = 0, max_cell_blocks: int = 0,
                 segments_per_warp: int = 0, segments_per_depth: int = 0):
        self.lib = load_library()
        self.lowered = lowered
        self._cm, self._keep = to_cmodel(lowered)
        tt = lowered.trace_target if trace_target is None else trace_target
        self.trace_target = np.ascontiguousarray(tt, dtype=np.int32)
        opt = COptions()
        opt.mode = mode
        opt.device = device
        opt.steps_per_launch = steps_per_launch
        opt.cells_per_block = cells_per_block
        opt.record_capacity_steps = record_capacity_steps
        opt.spike_capacity = spike_capacity
        opt.kernel_timing = 1 if kernel_timing else 0
        opt.codegen = codegen
        opt.max_cell_blocks = max_cell_blocks
        opt.segments_per_warp = segments_per_warp
        opt.segments_per_depth = segments_per_depth
        opt.n_trace = len(self.trace_target)
        opt.trace_target = self.trace_target.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)) if len(self.trace_target) else None
        self._opt = opt
        self.record_capacity_steps = record_capacity_steps
        self.spike_capacity = spike_capacity
        self.ctx = ctypes.c_void_p()
        rc = self.lib.edenGpuCreate(ctypes.byref(self._cm), ctypes.byref(opt), ctypes.byref(self.ctx))
        if rc != 0:
            msg = self._err()
            self.close()
            raise EdenGpuError(rc, msg)
        self.next_step = -3
        self.n_target = lowered.n_target

    def _err(self) -> str:
        if self.ctx:
            return self.lib.edenGpuLastError(self.ctx).decode()
        return "no context"

    def _check(self, rc: int):
        if rc != 0:
            raise EdenGpuError(rc, self._err())

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.edenGpuDestroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- stepping ------------------------------------------------------------
    def run_steps(self, n_steps: int) -> float:
        """Advance n_steps from the current step; returns device ms."""
        self._check(self.lib.edenGpuRun(self.ctx, ctypes.c_int64(self.next_step), ctypes.c_int64(n_steps)))
        self.next_step += n_steps
        return self.last_run_ms()

    def initialize(self):
        """The reference's four initialisation passes (steps -3..0)."""
        if self.next_step <= 0:
            self.run_steps(1 - self.next_step)

    def last_run_ms(self) -> float:
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        self._check(self.lib.edenGpuLastRunStats(self.ctx, ctypes.byref(ms), ctypes.byref(n)))
        self.last_launches = int(n.value)
        return float(ms.value)

    def fetch(self) -> Records:
        cap = self.record_capacity_steps
        nt = max(len(self.trace_target), 1)
        trace = np.zeros((cap, nt), np.float32)
        tstep = np.zeros(cap, np.int64)
        ssrc = np.zeros(self.spike_capacity, np.int32)
        sstep = np.zeros(self.spike_capacity, np.int64)
        stime = np.zeros(self.spike_capacity, np.float64)
        rec = CRecords()
        rec.trace = trace.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        rec.trace_step = tstep.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        rec.trace_capacity = cap
        rec.spike_src = ssrc.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        rec.spike_step = sstep.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        rec.spike_capacity = self.spike_capacity
        rec.spike_time_us = stime.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        self._check(self.lib.edenGpuFetchRecords(self.ctx, ctypes.byref(rec)))
        n, m = int(rec.n_trace_samples), int(rec.n_spikes)
        order = np.lexsort((ssrc[:m], sstep[:m]))
        return Records(trace[:n, :len(self.trace_target)].copy(), tstep[:n].copy(),
                       ssrc[:m][order].copy(), sstep[:m][order].copy(), stime[:m][order].copy())

    def run(self, n_steps: int | None = None, chunk: int | None = None) -> Records:
        """Initialise, then run n_steps non-initialisation steps (default: the
        model's length), fetching records between chunks."""
        if n_steps is None:
            n_steps = self.lowered.n_steps
        self.initialize()
        chunk = chunk or self.record_capacity_steps
        parts = []
        done = 0
        self.device_ms = 0.0
        self.launches = 0
        while done < n_steps:
            k = min(chunk, n_steps - done)
            self.device_ms += self.run_steps(k)
            self.launches += self.last_launches
            parts.append(self.fetch())
            done += k
        rec = Records(np.concatenate([p.trace for p in parts]) if parts else np.zeros((0, len(self.trace_target)), np.float32),
                      np.concatenate([p.trace_step for p in parts]) if parts else np.zeros(0, np.int64),
                      np.concatenate([p.spike_src for p in parts]) if parts else np.zeros(0, np.int32),
                      np.concatenate([p.spike_step for p in parts]) if parts else np.zeros(0, np.int64),
                      np.concatenate([p.spike_time for p in parts]) if parts else np.zeros(0, np.float64))
        # a spike in the final step would be logged at a step that never runs
        keep = rec.spike_step <= self.next_step - 1
        rec.spike_src, rec.spike_step, rec.spike_time = rec.spike_src[keep], rec.spike_step[keep], rec.spike_time[keep]
        return rec

    def kernel_stats(self) -> dict:
        """{kernel name: (total device ms, launches)} accumulated with kernel_timing."""
        out = {}
        for k, name in enumerate(KERNEL_NAMES):
            ms = ctypes.c_double()
            n = ctypes.c_int64()
            self._check(self.lib.edenGpuKernelStats(self.ctx, k, ctypes.byref(ms), ctypes.byref(n)))
            out[name] = (float(ms.value), int(n.value))
        return out

    def generated_source(self) -> str:
        """The CUDA source compiled for this model ('' when the built-in
        kernels run)."""
        n = self.lib.edenGpuGeneratedSource(self.ctx, None, 0)
        if n < 0:
            raise EdenGpuError(int(n), self._err())
        if n == 0:
            return ""
        buf = ctypes.create_string_buffer(int(n) + 1)
        self.lib.edenGpuGeneratedSource(self.ctx, buf, n + 1)
        return buf.value.decode()

    # -- state access ----------------------------------------------------------
    def read_v(self) -> np.ndarray:
        v = np.zeros(self.n_target, np.float32)
        self._check(self.lib.edenGpuReadV(self.ctx, _ptr(v), ctypes.c_int64(self.n_target)))
        return v

    def write_v(self, v: np.ndarray):
        v = np.ascontiguousarray(v, np.float32)
        self._check(self.lib.edenGpuWriteV(self.ctx, _ptr(v), ctypes.c_int64(self.n_target)))

    def fp64_cells(self) -> int:
        """Physical cells whose cable solve runs in double precision (those
        that can lose diagonal dominance; edenGpuFp64Cells)."""
        n = ctypes.c_int64()
        self._check(self.lib.edenGpuFp64Cells(self.ctx, ctypes.byref(n)))
        return n.value

    def read_synapses(self):
        n = len(self.lowered.syn_target)
        pend = np.zeros(max(n, 1), np.float32)
        a = np.zeros(max(n, 1), np.float32)
        b = np.zeros(max(n, 1), np.float32)
        self._check(self.lib.edenGpuReadSynapses(self.ctx, _ptr(pend), _ptr(a), _ptr(b), ctypes.c_int64(n)))
        return pend[:n], a[:n], b[:n]
