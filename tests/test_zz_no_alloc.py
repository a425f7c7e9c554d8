"""The adjoint entry point that allocates nothing, ``tam_fill_adjoint_static``.

Some callers cannot let a library call cudaMalloc or cudaFree while they
run: a solver that owns all device memory through its own pool or arena,
or a time-critical loop that must not pay the implicit device
synchronisation those calls bring.  For them the library has one variant of
the adjoint fill whose scratch is a fixed 64 MiB array compiled into the
library.  This file checks it through the C ABI against the allocating
entry point, ``tam_fill_adjoint``, on two calls in a row (the shared array
keeps the first call's contents), and checks its refusals.  It is collected
last so that a failure here comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from _helpers import nested_forest
from treeamr import (EvenParity, FieldSet, Forest, GhostSchedule, OddParity, Operators,
                     _native)
from treeamr.ghosts import DeviceSchedule

pytestmark = pytest.mark.gpu

TAM_EINVAL, TAM_EUNSUPPORTED = -1, -6
STATIC_BYTES = 64 << 20


ALL = (_native.TAM_STAGE_ALL_FIRST, _native.TAM_STAGE_ALL_LAST)


def _call(lib, ds, fn, y, nvars, factors, stages=ALL):
    stream = torch.cuda.current_stream()
    return fn(ds.handle, C.c_void_p(y.data_ptr()), nvars, y.shape[0],
              C.c_void_p(factors.data_ptr()), stages[0], stages[1],
              C.c_void_p(stream.cuda_stream))


def _fieldset(mesh, T):
    """``nested``: three levels, outer faces; ``walls``: 2^3 roots with low
    faces reflecting and high faces outflow, one root refined, a variable
    odd in each dimension, so the adjoint reads the factor table."""
    if mesh == "nested":
        return FieldSet(nested_forest(3, N=8), 2, G=2, T=T, device="cuda")
    f = Forest((2,) * 3, N=8, reflecting=((True, False),) * 3, outflow=((False, True),) * 3,
               extents=[(0.0, 2.0)] * 3)
    f.refine(f.leaves[0])
    f.balance()
    par = [(EvenParity,) * 3] + [tuple(OddParity if e == d else EvenParity for e in range(3))
                                  for d in range(3)]
    return FieldSet(f, len(par), G=2, T=T, parity=par, device="cuda")


@pytest.mark.parametrize("T", [np.float64, np.float32])
@pytest.mark.parametrize("mesh,stages", [("nested", ALL), ("walls", ALL), ("walls", (1, 1)),
                                         ("nested", (2, _native.TAM_STAGE_ALL_LAST))])
def test_static_adjoint_matches_allocating_adjoint(cuda_lib, T, mesh, stages):
    fs = _fieldset(mesh, T)
    sched = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    ds = DeviceSchedule(sched, 0)            # a fresh upload: no transposed stencils yet
    lib = cuda_lib
    y = torch.rand(fs.work.shape, dtype=fs.work.dtype, device="cuda")
    # refused before the set-up that allocates
    assert _call(lib, ds, lib.tam_fill_adjoint_static, y.clone(), fs.nvars, fs.factors) == TAM_EINVAL
    assert "tam_adjoint_scratch_bytes" in _native.last_error(ds.ctx)
    need = ds.adjoint_scratch_bytes(fs.nvars)       # set-up: builds the transposed stencils
    assert 0 < need <= STATIC_BYTES
    g = torch.Generator(device="cuda").manual_seed(17)
    for call in range(2):
        y0 = torch.empty(fs.work.shape, dtype=fs.work.dtype, device="cuda").uniform_(
            -1, 1, generator=g)
        expect = y0.clone()
        assert _call(lib, ds, lib.tam_fill_adjoint, expect, fs.nvars, fs.factors, stages) == 0
        got = y0.clone()
        rc = _call(lib, ds, lib.tam_fill_adjoint_static, got, fs.nvars, fs.factors, stages)
        assert rc == 0, _native.last_error(ds.ctx)
        torch.cuda.synchronize()
        # the same kernels in the same order: equal in every bit (tolerance 0)
        ib = torch.int64 if T == np.float64 else torch.int32
        assert torch.equal(got.view(ib), expect.view(ib)), f"call {call}"


def test_static_adjoint_refuses_oversized_scratch(cuda_lib):
    f = nested_forest(3, N=8)
    fs1 = FieldSet(f, 1, G=2, device="cuda")
    sched = GhostSchedule(fs1, Operators(prolongation=4, restriction=4))
    ds = DeviceSchedule(sched, 0)
    per_var = ds.adjoint_scratch_bytes(1)
    nvars = STATIC_BYTES // per_var + 1
    assert ds.adjoint_scratch_bytes(nvars) > STATIC_BYTES
    fs = FieldSet(f, nvars, G=2, device="cuda")
    rc = _call(cuda_lib, ds, cuda_lib.tam_fill_adjoint_static, fs.work, nvars, fs.factors)
    assert rc == TAM_EUNSUPPORTED
    assert "more than the built-in" in _native.last_error(ds.ctx)


def test_static_adjoint_refuses_a_turned_schedule(cuda_lib):
    """A schedule that turns transfers across a rotating seam needs the
    variable table, which only tam_fill_adjoint_ex takes."""
    from test_seam import quadrant_case
    quad, fs, s, *_ = quadrant_case(2, (1, 2), "none")
    fs.work, fs.factors = fs.work.cuda(), fs.factors.cuda()
    ds = DeviceSchedule(s, 0)
    ds.adjoint_scratch_bytes(fs.nvars)
    rc = _call(cuda_lib, ds, cuda_lib.tam_fill_adjoint_static, fs.work.clone(), fs.nvars,
               fs.factors)
    assert rc == TAM_EINVAL
    assert "variable table" in _native.last_error(ds.ctx)
