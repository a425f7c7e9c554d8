"""The state vector of an ODE integrator and its two copies to and from the
working array: ``statelength``, ``statevector``, ``statearray``,
``scatter``, ``gather`` (``src/state.jl:1-160``).

The state vector holds every block's own points only (``N + c_d`` per
dimension, every copy of a shared vertex-like point), in the working array's
index order minus the ghosts; a right-hand side scatters it into the working
array, fills the ghosts and writes its derivative in state layout.  Here the
copies are ``tam_scatter`` / ``tam_gather`` of libtreeamr_cuda.so, and
``scatter_fill`` is the scatter and the fill of one right-hand side.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, Optional

import numpy as np
import torch

from . import _native
from .ghosts import fill_ghosts
from .schedule import GhostSchedule
from .storage import FieldSet


def ownextents(fs: FieldSet):
    """``N + c_d`` per dimension (``src/storage.jl``, ``ownextents``)."""
    return tuple(fs.forest.N + cd for cd in fs.c)


def statelength(fs: FieldSet) -> int:
    """``prod(N + c_d) * nvars * nblocks`` (``src/state.jl:15-25``)."""
    return int(np.prod(ownextents(fs))) * fs.nvars * fs.nblocks()


def statevector(fs: FieldSet) -> torch.Tensor:
    """A zeroed state vector on the field set's device (``src/state.jl:27-43``)."""
    return torch.zeros(statelength(fs), dtype=fs.work.dtype, device=fs.work.device)


def statearray(u: torch.Tensor, fs: FieldSet) -> torch.Tensor:
    """``u`` viewed as ``(nblocks, nvars, O_D, ..., O_1)``, the working
    array's index order without the ghosts (``src/state.jl:45-57``)."""
    _check_length(u, fs)
    return u.view((fs.nblocks(), fs.nvars) + tuple(reversed(ownextents(fs))))


def _check_length(u: torch.Tensor, fs: FieldSet):
    if u.dim() != 1 or u.numel() != statelength(fs):
        raise ValueError(f"state vector has {u.numel()} entries but this field set needs "
                         f"{statelength(fs)}")


def _layout(fs: FieldSet) -> _native.tam_state_layout:
    L = _native.tam_state_layout()
    L.dtype = _native.TAM_F64 if fs.T == np.float64 else _native.TAM_F32
    L.ndim = fs.D
    own = ownextents(fs)
    for d in range(3):
        L.own[d] = own[d] if d < fs.D else 1
        L.stored[d] = fs.stored[d] if d < fs.D else 1
        L.ghosts[d] = fs.G[d] if d < fs.D else 0
    L.nvars = fs.nvars
    L.nblocks = fs.nblocks()
    return L


def _check(fs: FieldSet, u: torch.Tensor):
    _check_length(u, fs)
    if fs.work.device.type != "cuda" or u.device != fs.work.device:
        raise ValueError("the state vector and the working array must be on one CUDA device")
    if u.dtype != fs.work.dtype or not u.is_contiguous() or not fs.work.is_contiguous():
        raise ValueError("the state vector must be contiguous and of the working array's type")


def scatter(fs: FieldSet, u: torch.Tensor, stream: Optional[torch.cuda.Stream] = None) -> FieldSet:
    """Copy ``u`` into the working array's own points, ghosts untouched
    (``scatter!``, ``src/state.jl:130-141``)."""
    _check(fs, u)
    s = stream if stream is not None else torch.cuda.current_stream(fs.work.device)
    L = _layout(fs)
    rc = _native.lib().tam_scatter(C.byref(L), C.c_void_p(u.data_ptr()),
                                   C.c_void_p(fs.work.data_ptr()), C.c_void_p(s.cuda_stream))
    if rc != 0:
        raise _native.TamError(f"tam_scatter failed ({rc})")
    return fs


def gather(u: torch.Tensor, fs: FieldSet, stream: Optional[torch.cuda.Stream] = None) -> torch.Tensor:
    """Copy the working array's own points into ``u`` (``gather!``,
    ``src/state.jl:143-160``)."""
    _check(fs, u)
    s = stream if stream is not None else torch.cuda.current_stream(fs.work.device)
    L = _layout(fs)
    rc = _native.lib().tam_gather(C.byref(L), C.c_void_p(fs.work.data_ptr()),
                                  C.c_void_p(u.data_ptr()), C.c_void_p(s.cuda_stream))
    if rc != 0:
        raise _native.TamError(f"tam_gather failed ({rc})")
    return u


def scatter_fill(fs: FieldSet, schedule: GhostSchedule, u: torch.Tensor, *,
                 boundary: Optional[Callable] = None, method: str = "fused",
                 stream: Optional[torch.cuda.Stream] = None) -> FieldSet:
    """The first two steps of every right-hand side: ``scatter!(fs, u)``
    then ``fill_ghosts!(fs, schedule)`` (``src/state.jl:1-12``)."""
    scatter(fs, u, stream)
    return fill_ghosts(fs, schedule, boundary=boundary, method=method, stream=stream)
