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


_AVAILABLE: bool | None = None  # whether a CUDA device exists does not change within a process


def device() -> torch.device:
    global _AVAILABLE
    if _AVAILABLE is None:
        _AVAILABLE = torch.cuda.is_available()
    if not _AVAILABLE:
        raise RuntimeError("taichimps_gb300 runs on a CUDA device (GB300, sm_103a); none is available")
    return torch.device("cuda", torch.cuda.current_device())


_raw_stream = getattr(torch._C, "_cuda_getCurrentRawStream", None)


def stream() -> int:
    """The current stream of the current device as a cudaStream_t (a stream set by
    torch.cuda.stream() or a graph capture included)."""
    if _raw_stream is not None:
        return _raw_stream(torch.cuda.current_device())
    return torch.cuda.current_stream().cuda_stream


def lib():
    device()
    return _lib.load()


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def struct_buffer(st: ctypes.Structure) -> torch.Tensor:
    """A device byte buffer the size of a ctypes struct (zeroed)."""
    return torch.zeros(ctypes.sizeof(st), dtype=torch.uint8, device=device())


def _staged(raw: bytes) -> torch.Tensor:
    """`raw` in page-locked host memory.  PyTorch's pinned-memory cache keeps the block from reuse
    until the copies queued from it have run, so the caller need not wait for them."""
    h = torch.empty(len(raw), dtype=torch.uint8, pin_memory=True)
    ctypes.memmove(h.data_ptr(), raw, len(raw))
    return h


def push_struct(buf: torch.Tensor, st: ctypes.Structure) -> None:
    """Host struct -> device buffer, ordered on the current stream (the host does not wait)."""
    buf.copy_(_staged(bytes(st)), non_blocking=True)


def push_fields(buf: torch.Tensor, st: ctypes.Structure, first: str, last: str) -> None:
    """The fields `first` .. `last` (inclusive, in declaration order) of a host struct -> the same
    bytes of the device buffer, ordered on the current stream; the other bytes are left as the device
    has them."""
    cls = type(st)
    lo = getattr(cls, first).offset
    hi = getattr(cls, last).offset + getattr(cls, last).size
    buf[lo:hi].copy_(_staged(bytes(st)[lo:hi]), non_blocking=True)


def pull_struct(buf: torch.Tensor, cls: type[ctypes.Structure]) -> ctypes.Structure:
    """Device buffer -> host struct (synchronises the stream)."""
    return pull_many([(buf, cls)])[0]


def pull_many(items) -> list:
    """Several device buffers -> host values with one synchronisation: `items` holds (buffer, ctypes
    struct class) pairs, or (buffer, None) for the raw bytes as a numpy array."""
    sizes = [b.numel() * b.element_size() for b, _ in items]
    h = torch.empty(sum(sizes), dtype=torch.uint8, pin_memory=True)
    off = 0
    for (b, _), sz in zip(items, sizes):
        h[off:off + sz].copy_(b.reshape(-1).view(torch.uint8), non_blocking=True)
        off += sz
    torch.cuda.current_stream().synchronize()
    raw = h.numpy()
    out, off = [], 0
    for (b, cls), sz in zip(items, sizes):
        chunk = raw[off:off + sz]
        out.append(cls.from_buffer_copy(chunk.tobytes()) if cls is not None else chunk.copy())
        off += sz
    return out
