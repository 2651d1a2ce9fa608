"""A lowered model in one file, for hosts written in C or C++.

The file holds every field of `EdenGpuModel` (include/eden_gpu.h) under its
own name -- scalars as one-element arrays, pointer fields as the arrays they
point to, the channel and synapse type tables as the raw bytes of their C
structs -- plus the run's options and output layout: the recorded targets,
the step count, each trajectory column's scale from engine units to the
column's output units, and the event columns (spike source and selection id
of each).  `eden_gb300/host/eden_gpu_host.cpp` reads it and runs the
network through the C ABI, writing the reference's output files.

Layout: the 8-byte magic EDENGPU1, then records of
  u16 name length, name (ASCII), u8 type (0 int32, 1 int64, 2 float32,
  3 float64, 4 bytes), u64 element count, the elements (little-endian).
"""
from __future__ import annotations

import ctypes
import struct

import numpy as np

from .lowering import CModel, LoweredModel, to_cmodel

MAGIC = b"EDENGPU1"
_TYPES = {np.dtype(np.int32): 0, np.dtype(np.int64): 1, np.dtype(np.float32): 2, np.dtype(np.float64): 3}


def _record(f, name: str, arr) -> None:
    a = np.ascontiguousarray(arr)
    if a.dtype.fields is not None or a.dtype not in _TYPES:
        code, count, data = 4, a.nbytes, a.tobytes()
    else:
        code, count, data = _TYPES[a.dtype], a.size, a.astype(a.dtype.newbyteorder("<")).tobytes()
    nb = name.encode()
    f.write(struct.pack("<H", len(nb)) + nb + struct.pack("<BQ", code, count) + data)


def model_arrays(low: LoweredModel) -> dict:
    """name -> array for every field of EdenGpuModel, in declaration order."""
    cm, keep = to_cmodel(low)
    by_addr = {a.ctypes.data: a for a in keep}
    out = {}
    for name, ctype in CModel._fields_:
        val = getattr(cm, name)
        if ctype in (ctypes.c_int32, ctypes.c_int64, ctypes.c_float):
            dt = {ctypes.c_int32: np.int32, ctypes.c_int64: np.int64, ctypes.c_float: np.float32}[ctype]
            out[name] = np.array([val], dt)
            continue
        addr = ctypes.cast(val, ctypes.c_void_p).value
        if addr is None:
            continue  # an optional table left NULL (pois_rng_base)
        out[name] = by_addr[addr]
    return out


def write(path: str, low: LoweredModel, trace_target=None, trace_scale=None, event_src=None, event_id=None,
          n_steps: int | None = None, mode: int = 1) -> None:
    """Write `low` with its run options: recorded targets (default: the
    model's), their output scales (default 1e-3: mV to V), the event
    columns' sources and ids (default: every spike source, ids 0..n-1), the
    number of non-initialisation steps (default: the model's) and the
    execution mode (1 batched, 0 plain)."""
    tt = np.asarray(low.trace_target if trace_target is None else trace_target, np.int32)
    scale = np.full(len(tt), 1e-3) if trace_scale is None else np.asarray(trace_scale, np.float64)
    es = np.arange(len(low.src_target), dtype=np.int32) if event_src is None else np.asarray(event_src, np.int32)
    ids = [str(i) for i in range(len(es))] if event_id is None else [str(i) for i in event_id]
    with open(path, "wb") as f:
        f.write(MAGIC)
        for name, arr in model_arrays(low).items():
            _record(f, name, arr)
        _record(f, "run.trace_target", tt)
        _record(f, "run.trace_scale", scale)
        _record(f, "run.n_steps", np.array([low.n_steps if n_steps is None else n_steps], np.int64))
        _record(f, "run.mode", np.array([mode], np.int32))
        _record(f, "run.event_src", es)
        _record(f, "run.event_id", np.frombuffer("\n".join(ids).encode(), np.uint8))


def write_for_spec(path: str, spec, low: LoweredModel, mode: int = 1) -> None:
    """The same for a parsed LEMS simulation: its OutputFile columns (with
    each column's scale to its output units) and its first EventOutputFile's
    selections (spike source and id of each)."""
    scale = [c[3] for of in getattr(spec, "output_files", []) for c in of["cols"]]
    src, ids = [], []
    efs = getattr(spec, "event_files", [])
    if efs:
        off = spec.pop_offsets()
        for sid, _sel, (pop, idx) in efs[0]["sels"]:
            src.append(off[pop] + idx)
            ids.append(sid)
    write(path, low, trace_scale=np.asarray(scale, np.float64) if scale else None,
          event_src=np.asarray(src, np.int32), event_id=ids, mode=mode)


def read(path: str) -> dict:
    """name -> array of a file written by write() (byte records as uint8)."""
    codes = {0: np.int32, 1: np.int64, 2: np.float32, 3: np.float64, 4: np.uint8}
    out = {}
    with open(path, "rb") as f:
        if f.read(8) != MAGIC:
            raise ValueError(f"{path}: not a lowered-model file")
        while True:
            head = f.read(2)
            if len(head) < 2:
                break
            (n,) = struct.unpack("<H", head)
            name = f.read(n).decode()
            code, count = struct.unpack("<BQ", f.read(9))
            dt = np.dtype(codes[code]).newbyteorder("<")
            out[name] = np.frombuffer(f.read(count * dt.itemsize), dt).astype(codes[code])
    return out
