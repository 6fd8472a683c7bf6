"""Device plumbing: the CUDA device, the current stream, raw byte buffers."""

from __future__ import annotations

import ctypes
import gc

import numpy as np
import torch

from . import _lib


def capture_graph(launch) -> torch.cuda.CUDAGraph:
    """Captures what `launch()` enqueues on the current stream into a CUDA graph (on a side
    stream).  Python's cyclic garbage collector is held off during the capture: a collection
    inside it could destroy an unreferenced graph of an earlier run, a call CUDA does not
    permit while a stream is capturing (the capture would be invalidated)."""
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    enabled = gc.isenabled()
    gc.disable()
    try:
        with torch.cuda.graph(g, stream=side):
            launch()
    finally:
        if enabled:
            gc.enable()
    torch.cuda.current_stream().wait_stream(side)
    return g


# Optional per-launch CUDA-event timing, keyed by kernel name; None when off.
# bench.py turns it on for the kernels whose roofline it reports.
TIMED: dict[str, list] | None = None


class timed:
    """Record CUDA events around one launch when ``TIMED`` collects `name`."""

    def __init__(self, name: str):
        self.name = name
        self.on = TIMED is not None and name in TIMED

    def __enter__(self):
        if self.on:
            self.e0 = torch.cuda.Event(enable_timing=True)
            self.e0.record()
        return self

    def __exit__(self, *exc):
        if self.on:
            e1 = torch.cuda.Event(enable_timing=True)
            e1.record()
            TIMED[self.name].append((self.e0, e1))
        return False


def device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("taichimps_gb300 runs on a CUDA device (GB300, sm_103a); none is available")
    return torch.device("cuda", torch.cuda.current_device())


def stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def lib():
    device()
    return _lib.load()


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def struct_buffer(st: ctypes.Structure) -> torch.Tensor:
    """A device byte buffer the size of a ctypes struct (zeroed)."""
    return torch.zeros(ctypes.sizeof(st), dtype=torch.uint8, device=device())


def push_struct(buf: torch.Tensor, st: ctypes.Structure) -> None:
    """Host struct -> device buffer, ordered on the current stream."""
    raw = np.frombuffer(bytes(st), dtype=np.uint8).copy()
    buf.copy_(torch.from_numpy(raw), non_blocking=False)


def pull_struct(buf: torch.Tensor, cls: type[ctypes.Structure]) -> ctypes.Structure:
    """Device buffer -> host struct (synchronises the stream)."""
    raw = buf.cpu().numpy().tobytes()
    return cls.from_buffer_copy(raw)
