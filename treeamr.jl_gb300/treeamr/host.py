"""Ghost fills of field states held in host memory (``tam_fill_host``).

The reference fills host arrays in place (``fill_ghosts!``,
``src/ghosts.jl:1783``).  Here a host-resident state is uploaded, filled on
the GPU and downloaded, all asynchronous on one stream.  ``HostPipeline``
keeps ``depth`` streams, each with its own device buffer, and gives
consecutive states to them in turn, so one state's upload, another's fill
and a third's download run together: the copy engines in both directions
and the SMs stay busy at once.

With ``own=True`` only what the fill reads goes up: the own points, read
by a kernel straight from the page-locked host buffer
(``tam_fill_host_own``); the filled array comes back whole.  That needs a
schedule that writes every point outside the own boxes (no outer-face hook
regions), since the rest of the device buffer is not uploaded.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional

import torch

from . import _native
from .ghosts import check_fill, device_schedule
from .schedule import GhostSchedule
from .storage import FieldSet


class HostPipeline:
    """Round-robin host fills of the states of one field set's shape.

    ``fs`` gives the shape, element type, factor table and device; its own
    ``work`` is not touched.  Host buffers should be page-locked
    (``Tensor.pin_memory()``), or the copies do not overlap other work."""

    def __init__(self, fs: FieldSet, schedule: GhostSchedule, depth: int = 3,
                 own: bool = False):
        if depth < 1:
            raise ValueError("depth must be at least 1")
        check_fill(fs, schedule)
        if own and schedule.boundaries:
            raise ValueError("own-point uploads need a schedule that writes every point outside "
                             "the own boxes, and this one leaves outer-face regions to a hook")
        self.own = own
        if own:
            from .state import _layout
            self.layout = _layout(fs)
        self.fs = fs
        self.device = fs.work.device
        self.ds = device_schedule(schedule, self.device.index or 0)
        self.streams: List[torch.cuda.Stream] = [torch.cuda.Stream(self.device)
                                                 for _ in range(depth)]
        self.buffers = [torch.empty_like(fs.work) for _ in range(depth)]
        self.next = 0

    def submit(self, host_in: torch.Tensor, host_out: Optional[torch.Tensor] = None) -> int:
        """Fill the state in ``host_in`` into ``host_out`` (default: in place);
        returns the slot used.  Asynchronous: the host buffers must stay
        untouched until ``synchronize`` (or the slot's stream) says so."""
        host_out = host_in if host_out is None else host_out
        for t in (host_in, host_out):
            if t.device.type != "cpu" or not t.is_contiguous() or t.shape != self.fs.work.shape \
                    or t.dtype != self.fs.work.dtype:
                raise ValueError("host buffers must be contiguous CPU tensors of the field's "
                                 "shape and element type")
        k = self.next
        self.next = (k + 1) % len(self.streams)
        st = self.streams[k]
        if self.own:
            rc = self.ds.lib.tam_fill_host_own(
                self.ds.handle, C.byref(self.layout), C.c_void_p(host_in.data_ptr()),
                C.c_void_p(host_out.data_ptr()), C.c_void_p(self.buffers[k].data_ptr()),
                self.fs.nvars, self.fs.nblocks(), C.c_void_p(self.fs.factors.data_ptr()),
                _native.TAM_STAGE_ALL_FIRST, _native.TAM_STAGE_ALL_LAST,
                C.c_void_p(st.cuda_stream))
            _native.check(rc, self.ds.ctx, "tam_fill_host_own")
            return k
        rc = self.ds.lib.tam_fill_host(
            self.ds.handle, C.c_void_p(host_in.data_ptr()), C.c_void_p(host_out.data_ptr()),
            C.c_void_p(self.buffers[k].data_ptr()), self.fs.nvars, self.fs.nblocks(),
            C.c_void_p(self.fs.factors.data_ptr()), _native.TAM_STAGE_ALL_FIRST,
            _native.TAM_STAGE_ALL_LAST, C.c_void_p(st.cuda_stream))
        _native.check(rc, self.ds.ctx, "tam_fill_host")
        return k

    def own_bytes(self) -> int:
        """Bytes an own-point upload moves per state."""
        import numpy as np
        n = self.fs.nvars * self.fs.nblocks() * self.fs.T.itemsize
        for d in range(self.fs.D):
            n *= self.fs.forest.N + self.fs.c[d]
        return int(n)

    def wait_on(self, stream: torch.cuda.Stream):
        """Make every slot's stream wait for what ``stream`` has queued."""
        for st in self.streams:
            st.wait_stream(stream)

    def join(self, stream: torch.cuda.Stream):
        """Make ``stream`` wait for every slot's queued work."""
        for st in self.streams:
            stream.wait_stream(st)

    def synchronize(self):
        for st in self.streams:
            st.synchronize()
