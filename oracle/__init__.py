"""The oracle: a CPU restatement of the reference's ghost fill.

TEST INFRASTRUCTURE ONLY -- imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py's cpu_baseline leg.  The product never calls it.

``fill(schedule, work, ...)`` and ``fill_adjoint(...)`` run ``fill_oracle.c``
(compiled by ``build()`` into ``oracle/_build``) over the same flattened
schedule the CUDA library uploads; ``exact_weights`` and friends are in the
host package's ``operators`` module and are pinned by the reference's
known-answer tests in ``tests/test_operators.py``.

Parity status: pinned by the reference's known-answer and property tests
(restated in tests/), and by a second oracle independent of the product's
schedule (``oracle/pointwise.py``, ``pointwise.c``): the meshes rebuilt from
their construction rules and every ghost derived point by point from the
forest's geometry, equal to this replay bit for bit.  No golden vectors exist
in the reference and the reference (Julia) cannot run in this environment.
What this replay takes from the product: the flattened schedule (which
transfer writes which ghost, windows, weights, stage order).  What the
point-by-point oracle takes from it: the forest's leaves and their order
(checked against a rebuild and the curve order), the field layout and the
parity table's meaning, nothing else.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libtam_oracle.so")
SRC = os.path.join(HERE, "fill_oracle.c")
HDR = os.path.join(ROOT, "include", "treeamr_cuda.h")

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """gcc -O2 -fopenmp -ffp-contract=off: no fused multiply-add on any host."""
    with _lock:
        os.makedirs(BUILD_DIR, exist_ok=True)
        newest = max(os.path.getmtime(SRC), os.path.getmtime(HDR))
        fresh = not force and os.path.exists(LIB_PATH) and \
            os.path.getmtime(LIB_PATH) >= newest
        if not fresh:
            tmp = LIB_PATH + ".tmp"
            cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
                   "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"), SRC, "-o", tmp]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"oracle build failed:\n{r.stderr}")
            os.replace(tmp, LIB_PATH)
    from . import pointwise
    pointwise.build(force)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        l = C.CDLL(LIB_PATH)
        l.oracle_fill.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                  C.c_int32, C.c_int, C.c_int]
        l.oracle_fill.restype = C.c_int
        l.oracle_fill_turned.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                         C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int,
                                         C.c_int]
        l.oracle_fill_turned.restype = C.c_int
        l.oracle_fill_adjoint.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                          C.c_int32, C.c_int32]
        l.oracle_fill_adjoint.restype = C.c_int
        l.oracle_fill_adjoint_turned.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                                 C.c_void_p, C.c_int32, C.c_int32]
        l.oracle_fill_adjoint_turned.restype = C.c_int
        l.oracle_fill_adjoint_pair.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                               C.c_void_p, C.c_void_p, C.c_int32, C.c_int32]
        l.oracle_fill_adjoint_pair.restype = C.c_int
        _lib = l
    return _lib


def _descriptor(schedule):
    import treeamr._native as nat
    cache = schedule.__dict__.setdefault("_oracle_desc", None)
    if cache is None:
        cache = nat.Descriptor(schedule)
        schedule._oracle_desc = cache
    return cache


ALL_FIRST, ALL_LAST = -1, 0x7FFFFFFF


def fill(schedule, work: np.ndarray, nvars: int, factors: np.ndarray, *, first=ALL_FIRST,
         last=ALL_LAST, nthreads: int = 1, one_tap: bool = True, rotvars=None,
         alt: np.ndarray = None) -> np.ndarray:
    """In place on ``work`` (shape (nblocks, nvars, S_D..S_1), C order).

    ``one_tap`` picks the form of the stencil sum (src/ghosts.jl:28-56): the
    reference's CPU form, where a dimension whose weight column has a single
    nonzero weight takes only that tap, or (False) its device form, the full
    sum.  They differ only where a NaN or an infinity sits under a zero
    weight.  A schedule that turns transfers across a seam reads the field
    set's variable table ``rotvars`` (nvars x 4, 1-based) and, for an odd
    orientation, ``alt`` (default ``work``)."""
    assert work.flags.c_contiguous and work.dtype == np.dtype(schedule.T)
    d = _descriptor(schedule)
    f = np.ascontiguousarray(np.asfortranarray(factors).ravel(order="F"), dtype=work.dtype)
    if rotvars is None:
        rc = lib().oracle_fill(C.addressof(d.desc), work.ctypes.data, nvars, f.ctypes.data,
                               first, last, nthreads, 1 if one_tap else 0)
    else:
        rv = np.ascontiguousarray(np.asfortranarray(rotvars).ravel(order="F"), dtype=np.int32)
        a = work if alt is None else alt
        # a RotationPair partner holds the swapped layout: as many points a block
        assert a.flags.c_contiguous and a.size == work.size and a.dtype == work.dtype
        rc = lib().oracle_fill_turned(C.addressof(d.desc), work.ctypes.data, a.ctypes.data,
                                      nvars, f.ctypes.data, rv.ctypes.data, first, last,
                                      nthreads, 1 if one_tap else 0)
    if rc != 0:
        raise RuntimeError("oracle_fill failed (a turned schedule needs rotvars)")
    return work


def fill_adjoint(schedule, y: np.ndarray, nvars: int, factors: np.ndarray, *, first=ALL_FIRST,
                 last=ALL_LAST, rotvars=None, alt: np.ndarray = None) -> np.ndarray:
    """In place on ``y``: the scatter-form transpose of ``fill``; with ``alt``
    (a RotationPair partner's cotangent, in the partner's layout) odd turns
    scatter onto ``alt``."""
    assert y.flags.c_contiguous and y.dtype == np.dtype(schedule.T)
    d = _descriptor(schedule)
    f = np.ascontiguousarray(np.asfortranarray(factors).ravel(order="F"), dtype=y.dtype)
    rv = None if rotvars is None else \
        np.ascontiguousarray(np.asfortranarray(rotvars).ravel(order="F"), dtype=np.int32)
    if alt is not None:
        assert alt.flags.c_contiguous and alt.size == y.size and alt.dtype == y.dtype
        rc = lib().oracle_fill_adjoint_pair(C.addressof(d.desc), y.ctypes.data, alt.ctypes.data,
                                            nvars, f.ctypes.data,
                                            None if rv is None else rv.ctypes.data, first, last)
    else:
        rc = lib().oracle_fill_adjoint_turned(C.addressof(d.desc), y.ctypes.data, nvars,
                                              f.ctypes.data,
                                              None if rv is None else rv.ctypes.data, first, last)
    if rc != 0:
        raise RuntimeError("oracle_fill_adjoint failed")
    return y


def fill_fieldset(fs, schedule, *, boundary_values=None, nthreads: int = 1,
                  one_tap: bool = True) -> np.ndarray:
    """The oracle's fill of a field set's current contents, returned as a new
    host array; ``boundary_values(host, fs, regions)`` fills the outer-face
    regions between phase 1 and the prolongations."""
    host = fs.work.detach().cpu().numpy().copy()
    rv = getattr(fs, "rotvars_host", None)
    if boundary_values is None or not schedule.boundaries:
        return fill(schedule, host, fs.nvars, fs.factors_host, nthreads=nthreads,
                    one_tap=one_tap, rotvars=rv)
    fill(schedule, host, fs.nvars, fs.factors_host, last=1, nthreads=nthreads, one_tap=one_tap,
         rotvars=rv)
    boundary_values(host, fs, schedule.boundaries)
    return fill(schedule, host, fs.nvars, fs.factors_host, first=2, nthreads=nthreads,
                one_tap=one_tap, rotvars=rv)


def _own_slices(fs):
    """Own range ``G_d+1 : G_d+N+c_d`` per dimension, in the host array's
    reversed index order."""
    N = fs.forest.N
    return tuple(slice(g, g + N + cd) for g, cd in reversed(list(zip(fs.G, fs.c))))


def scatter(fs, work: np.ndarray, u: np.ndarray) -> np.ndarray:
    """``scatter!`` (src/state.jl:101-106, 130-141): the state vector's
    entries, in the working array's order without ghosts, into the own
    points of ``work`` (shape (nblocks, nvars, S_D..S_1)); ghosts untouched."""
    own = _own_slices(fs)
    shape = work[(slice(None), slice(None)) + own].shape
    work[(slice(None), slice(None)) + own] = u.reshape(shape)
    return work


def gather(fs, work: np.ndarray) -> np.ndarray:
    """``gather!`` (src/state.jl:108-113, 143-160): the own points of ``work``
    as a flat state vector."""
    own = _own_slices(fs)
    return np.ascontiguousarray(work[(slice(None), slice(None)) + own]).ravel()


def cell_boundary(fs, host: np.ndarray, regions, g) -> np.ndarray:
    """The device hook's built-in functions evaluated on the host, in place on
    ``host``: every point of every region gets ``g(x, v)``, ``x`` the exactly
    rounded ``nodeposition`` (``src/storage.jl:1008-1017``, through
    ``FieldSet.positions``), a polynomial's terms ``((c * x1^a) * x2^b) *
    x3^c`` with powers by repeated multiplication, summed in order from +0,
    every operation rounded once in the element type.  ``Relative(f)``
    (``src/ghosts.jl:1431-1475``): ``f(x_g) + (u(r) - f(x_r))`` with ``r`` the
    region's clamped index, read from ``host``."""
    from treeamr.boundary import Constant, Relative
    T = np.dtype(fs.T).type
    D = fs.D
    relative = isinstance(g, Relative)
    f = g.f if relative else g

    def ev(x, v):
        if isinstance(f, Constant):
            return T(f.values[v])
        val = T(0)
        for exps, coefs in f.terms:
            term = T(coefs[v])
            for d, e in enumerate(exps):
                for _ in range(e):
                    term = T(term * x[d])
            val = T(val + term)
        return val

    for r in regions:
        pos = fs.positions(r.block)
        idxs = [range(a, z + 1) for a, z in r.region]
        for I in np.ndindex(*[len(i) for i in idxs]):
            idx = tuple(idxs[d][I[d]] for d in range(D))
            x = [T(pos[d][idx[d] - 1]) for d in range(D)]
            rr = tuple((r.clamps[d] if r.clamps and r.clamps[d] else idx[d]) for d in range(D))
            xr = [T(pos[d][rr[d] - 1]) for d in range(D)]
            for v in range(fs.nvars):
                val = ev(x, v)
                if relative:
                    ur = T(host[(r.block, v) + tuple(i - 1 for i in reversed(rr))])
                    val = T(val + T(ur - ev(xr, v)))
                host[(r.block, v) + tuple(i - 1 for i in reversed(idx))] = val
    return host


def axis_project(schedule, host: np.ndarray, nvars: int, factors: np.ndarray,
                 rotvars: np.ndarray) -> np.ndarray:
    """A seam's axis projection on the host, in place (``axis_project!``,
    ``mean_gather_kernel!`` in its paired form, src/ghosts.jl:599-660,
    736-770): each axis point's variable ``v`` becomes
    ``((t_0 + t_2) + (t_1 + t_3)) / 4`` (a half turn: ``(t_0 + t_2) / 2``) with
    ``t_r = factors[v, 3^D r] * u[rotvars[v, r] - 1]`` (``t_0 = u[v]``), every
    mean gathered before any is written, in the element type."""
    pts, orbit = schedule.axis, schedule.axis_orbit
    if not pts:
        return host
    T = host.dtype.type
    D = schedule.forest.D
    ncol = 3 ** D
    M = len(orbit)
    means = []
    for b, idx in pts:
        at = tuple(i - 1 for i in reversed(idx))
        vals = []
        for v in range(nvars):
            def term(r):
                if r == 0:
                    return T(host[(b, v) + at])
                sv = int(rotvars[v, r]) - 1
                return T(T(factors[v, ncol * r]) * T(host[(b, sv) + at]))
            acc = T(term(orbit[0]) + term(orbit[1]))
            if M == 4:
                acc = T(acc + T(term(orbit[2]) + term(orbit[3])))
            vals.append(T(acc / T(M)))
        means.append(vals)
    for (b, idx), vals in zip(pts, means):
        at = tuple(i - 1 for i in reversed(idx))
        for v in range(nvars):
            host[(b, v) + at] = vals[v]
    return host


def axis_project_adjoint(schedule, host: np.ndarray, nvars: int, factors: np.ndarray,
                         rotvars: np.ndarray) -> np.ndarray:
    """The transpose of ``axis_project``, in place, in scatter form: the
    projection's mean for variable ``v`` read ``factors[v, 3^D r] *
    u[rotvars[v, r] - 1]`` over the orbit, so ``y[v] / M`` times that factor
    is added back onto variable ``rotvars[v, r] - 1`` (``v`` itself for
    ``r = 0``), summed in float64.  The reference has no adjoint; this is the
    transpose of ``axis_project!`` (src/ghosts.jl:599-660)."""
    pts, orbit = schedule.axis, schedule.axis_orbit
    if not pts:
        return host
    D = schedule.forest.D
    ncol = 3 ** D
    M = len(orbit)
    outs = []
    for b, idx in pts:
        at = tuple(i - 1 for i in reversed(idx))
        yv = [float(host[(b, v) + at]) for v in range(nvars)]
        out = [0.0] * nvars
        for v in range(nvars):
            for r in orbit:
                sv = v if r == 0 else int(rotvars[v, r]) - 1
                f = 1.0 if r == 0 else float(factors[v, ncol * r])
                out[sv] += f * yv[v] / M
        outs.append(out)
    for (b, idx), out in zip(pts, outs):
        at = tuple(i - 1 for i in reversed(idx))
        for v in range(nvars):
            host[(b, v) + at] = out[v]
    return host
