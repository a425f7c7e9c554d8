"""RK4 for the wave equation over a batch of forests, forward and adjoint.

The reference's wave test (``test/wave.jl:49-110,178-200``) advances
``u_t = v, v_t = lap(u)`` with classical RK4, each stage a ghost fill and the
7-point Laplacian on owned points.  ``WaveSolver`` does that for every forest
of a ``ForestBatch`` at once:

* every stage is one batched fill (``tam_batch_fill``) and one batched
  right-hand side (``tam_wave_rhs``), and a whole step can be captured in a
  CUDA graph and replayed;
* the backward pass is the discrete adjoint of the same steps, each stage's
  transpose being the right-hand side's transpose and then the fill's
  (``tam_batch_fill_adjoint``).  The dynamics are linear, so states are needed
  only for a loss that reads every step; they are recomputed from
  checkpoints every ``checkpoint`` steps.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, Optional

import numpy as np
import torch

from . import _native
from .batch import ForestBatch

_WAVE_BLOCK = np.dtype([("off", np.int64), ("S", np.int32, (3,)), ("G", np.int32),
                        ("N", np.int32), ("pad", np.int32), ("inv_h2", np.float64)])
assert _WAVE_BLOCK.itemsize == 40


class WaveSolver:
    """The state is the batch's arena layout with variables (u, v)."""

    def __init__(self, batch: ForestBatch, dt: Optional[float] = None, cfl: float = 0.25):
        if batch.nvars != 2 or batch.D != 3:
            raise ValueError("the wave solver needs 3-D field sets with two variables (u, v)")
        rows = []
        hmin = np.inf
        for m, fs in enumerate(batch.fieldsets):
            if any(cd != 0 for cd in fs.c) or min(fs.G) < 1:
                raise ValueError("the wave right-hand side is for cell-centred sets with G >= 1")
            f = fs.forest
            S = fs.stored
            per_block = fs.nvars * S[0] * S[1] * S[2]
            for b, k in enumerate(f.leaves):
                h = float(f.spacing(k.level, np.float64))
                hmin = min(hmin, h)
                rows.append((batch.offsets[m] + b * per_block, S, fs.G[0], f.N, 0, 1.0 / (h * h)))
        table = np.zeros(len(rows), dtype=_WAVE_BLOCK)
        for i, r in enumerate(rows):
            table[i] = r
        self.nblocks = len(rows)
        self.max_points = int(max(np.prod(fs.stored) for fs in batch.fieldsets))
        self.table = torch.from_numpy(table.view(np.uint8).copy()).to(batch.device)
        self.batch = batch
        self.lib = _native.lib()
        self.lib.tam_wave_rhs.argtypes = [C.c_int32, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p,
                                          C.c_void_p, C.c_int32, C.c_void_p]
        self.lib.tam_wave_rhs.restype = C.c_int
        self.lib.tam_wave_rk4_stage.argtypes = [C.c_int32, C.c_void_p, C.c_int32, C.c_int32,
                                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_double, C.c_double, C.c_void_p]
        self.lib.tam_wave_rk4_stage.restype = C.c_int
        self.lib.tam_wave_rk4_adjoint_stage.argtypes = [C.c_int32, C.c_void_p, C.c_int32,
                                                        C.c_int32, C.c_void_p, C.c_double,
                                                        C.c_void_p, C.c_double, C.c_void_p,
                                                        C.c_void_p, C.c_void_p]
        self.lib.tam_wave_rk4_adjoint_stage.restype = C.c_int
        self.dtype_code = _native.TAM_F64 if batch.T == np.float64 else _native.TAM_F32
        self.dt = float(dt) if dt is not None else cfl * hmin
        like = batch.arena
        self.k = [torch.zeros_like(like) for _ in range(4)]
        self.tmp = torch.zeros_like(like)
        self.adj = [torch.zeros_like(like) for _ in range(3)]

    # -- the pieces ------------------------------------------------------------
    def rhs(self, x: torch.Tensor, out: torch.Tensor, adjoint: bool = False):
        s = torch.cuda.current_stream(x.device)
        rc = self.lib.tam_wave_rhs(self.dtype_code, C.c_void_p(self.table.data_ptr()),
                                   self.nblocks, self.max_points, C.c_void_p(x.data_ptr()),
                                   C.c_void_p(out.data_ptr()), 1 if adjoint else 0,
                                   C.c_void_p(s.cuda_stream))
        if rc != 0:
            raise _native.TamError(f"tam_wave_rhs failed ({rc})")
        return out

    def stage(self, x: torch.Tensor, y: torch.Tensor, t_out: Optional[torch.Tensor],
              acc_in: Optional[torch.Tensor], acc_out: torch.Tensor, ct: float, ca: float):
        """One fused RK4 stage (``tam_wave_rk4_stage``): with k = R(x),
        ``t_out = y + ct k`` and ``acc_out = (acc_in or y) + ca k``."""
        s = torch.cuda.current_stream(x.device)
        ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
        rc = self.lib.tam_wave_rk4_stage(self.dtype_code, C.c_void_p(self.table.data_ptr()),
                                         self.nblocks, self.max_points, ptr(x), ptr(y),
                                         ptr(t_out), ptr(acc_in), ptr(acc_out), float(ct),
                                         float(ca), C.c_void_p(s.cuda_stream))
        if rc != 0:
            raise _native.TamError(f"tam_wave_rk4_stage failed ({rc})")

    def stage_adjoint(self, g: torch.Tensor, c1: float, xprev: Optional[torch.Tensor],
                      c2: float, out: torch.Tensor, ybar: Optional[torch.Tensor]):
        """``out = R^T (c1 g + c2 xprev)`` and ``ybar += xprev``
        (``tam_wave_rk4_adjoint_stage``)."""
        s = torch.cuda.current_stream(g.device)
        ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
        rc = self.lib.tam_wave_rk4_adjoint_stage(
            self.dtype_code, C.c_void_p(self.table.data_ptr()), self.nblocks, self.max_points,
            ptr(g), float(c1), ptr(xprev), float(c2), ptr(out), ptr(ybar),
            C.c_void_p(s.cuda_stream))
        if rc != 0:
            raise _native.TamError(f"tam_wave_rk4_adjoint_stage failed ({rc})")

    def F(self, x: torch.Tensor, out: torch.Tensor):
        """``out = R(A x)``; ``x``'s ghosts are filled in place."""
        self.batch.fill(x)
        return self.rhs(x, out)

    def FT(self, kbar: torch.Tensor, out: torch.Tensor):
        """``out = A^T R^T kbar``."""
        self.rhs(kbar, out, adjoint=True)
        self.batch.fill_adjoint(out)
        return out

    # -- forward ---------------------------------------------------------------
    def step(self, y: torch.Tensor):
        """One RK4 step of ``y`` in place: four fills, each followed by one
        fused stage that forms the next stage state and adds the stage's
        share of the step, k1/6 + k2/3 + k3/3 + k4/6 times dt, in that order."""
        dt = self.dt
        ta, tb, acc = self.k[0], self.k[1], self.k[2]
        self.batch.fill(y)
        self.stage(y, y, ta, None, acc, dt / 2, dt / 6)
        self.batch.fill(ta)
        self.stage(ta, y, tb, acc, acc, dt / 2, dt / 3)
        self.batch.fill(tb)
        self.stage(tb, y, ta, acc, acc, dt, dt / 3)
        self.batch.fill(ta)
        self.stage(ta, y, None, acc, y, 0.0, dt / 6)
        return y

    def capture(self, y: torch.Tensor, steps: int = 1) -> torch.cuda.CUDAGraph:
        """A CUDA graph of ``steps`` RK4 steps of ``y`` (warmed up first: the
        fills and right-hand sides allocate nothing)."""
        side = torch.cuda.Stream(device=y.device)
        side.wait_stream(torch.cuda.current_stream(y.device))
        with torch.cuda.stream(side):
            probe = y.clone()
            self.step(probe)
        torch.cuda.current_stream(y.device).wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            for _ in range(steps):
                self.step(y)
        return g

    def native_graph(self, y: torch.Tensor, steps: int = 1) -> "NativeGraph":
        """The same ``steps`` RK4 steps of ``y`` captured by the library
        (``tam_graph_capture_rk4``); ``launch()`` replays them."""
        ta, tb, acc = self.k[0], self.k[1], self.k[2]
        b = self.batch
        if b.rotvars is not None or b.axis_members:
            raise ValueError("the library's RK4 graph fills with tam_batch_fill, which turns no "
                             "ghosts across a seam: capture() the batch's own fills instead")
        h = C.c_void_p()
        rc = self.lib.tam_graph_capture_rk4(
            b.handle, self.dtype_code, C.c_void_p(self.table.data_ptr()), self.nblocks,
            self.max_points, C.c_void_p(y.data_ptr()), C.c_void_p(ta.data_ptr()),
            C.c_void_p(tb.data_ptr()), C.c_void_p(acc.data_ptr()), y.numel(), b.nvars,
            C.c_void_p(b.factor_arena.data_ptr()), b.factor_arena.numel(), float(self.dt),
            steps, y.device.index or 0, C.byref(h))
        if rc != 0:
            raise _native.TamError(f"tam_graph_capture_rk4 failed ({rc})")
        return NativeGraph(self.lib, h, (y, ta, tb, acc, self.table, b))

    # -- the adjoint -------------------------------------------------------------
    #
    # One step as the forward runs it, with P the fill (applied in place) and
    # R the right-hand side:  z = P y;  k1 = R z;  x2 = z + dt/2 k1, k2 = R P x2;
    # x3 = z + dt/2 k2, k3 = R P x3;  x4 = z + dt k3, k4 = R P x4;
    # y' = z + dt/6 k1 + dt/3 k2 + dt/3 k3 + dt/6 k4.  Its transpose, from g = y'bar:
    # zbar = g; each k_ibar starts at its weight times g; x4bar = P^T R^T k4bar
    # adds to zbar and (times dt) to k3bar; x3bar and x2bar likewise (times
    # dt/2) to k2bar and k1bar; R^T k1bar adds to zbar; ybar = P^T zbar.
    def step_adjoint(self, ybar: torch.Tensor):
        """``ybar <- M^T ybar`` for one RK4 step ``M``, in place.  Each stage's
        cotangent k_ibar = w_i g + c x_(i+1)bar is formed inside the transposed
        right-hand side, which also adds the previous stage's x bar to
        ``ybar``."""
        dt = self.dt
        g, xa, xb = self.adj
        g.copy_(ybar)
        self.stage_adjoint(g, dt / 6, None, 0.0, xa, None)         # x4bar = P^T R^T k4bar
        self.batch.fill_adjoint(xa)
        self.stage_adjoint(g, dt / 3, xa, dt, xb, ybar)            # x3bar; ybar += x4bar
        self.batch.fill_adjoint(xb)
        self.stage_adjoint(g, dt / 3, xb, dt / 2, xa, ybar)        # x2bar; ybar += x3bar
        self.batch.fill_adjoint(xa)
        self.stage_adjoint(g, dt / 6, xa, dt / 2, xb, ybar)        # R^T k1bar; ybar += x2bar
        ybar.add_(xb)
        self.batch.fill_adjoint(ybar)
        return ybar

    def run(self, y: torch.Tensor, steps: int, checkpoint: int = 0):
        """``steps`` forward steps of ``y`` in place; with ``checkpoint`` > 0, the
        states at every ``checkpoint``-th step (from step 0) are kept."""
        saved = {}
        for n in range(steps):
            if checkpoint and n % checkpoint == 0:
                saved[n] = y.clone()
            self.step(y)
        return saved

    def gradient(self, y0: torch.Tensor, steps: int, dloss: Callable, checkpoint: int = 2):
        """The gradient with respect to ``y0`` of ``L = sum_n l(y_n)``, n = 1..steps,
        given ``dloss(y) = dl/dy``: the states are recomputed from checkpoints
        every ``checkpoint`` steps during the backward sweep."""
        y = y0.clone()
        saved = self.run(y, steps, checkpoint)
        ybar = torch.zeros_like(y0)
        cur, cur_n = None, None
        for n in range(steps, 0, -1):
            # y_n: from the latest checkpoint at or below n-1, stepped forward
            c = ((n - 1) // checkpoint) * checkpoint
            cur = saved[c].clone()
            for _ in range(n - c):
                self.step(cur)
            ybar.add_(dloss(cur))
            self.step_adjoint(ybar)
        return ybar


class NativeGraph:
    """A graph of RK4 steps captured by the library; keeps what it reads
    alive and frees the graph with itself."""

    def __init__(self, lib, handle, keep):
        self.lib, self.handle, self._keep = lib, handle, keep

    def launch(self, stream: Optional[torch.cuda.Stream] = None):
        s = stream if stream is not None else torch.cuda.current_stream(self._keep[0].device)
        rc = self.lib.tam_graph_launch(self.handle, C.c_void_p(s.cuda_stream))
        if rc != 0:
            raise _native.TamError(f"tam_graph_launch failed ({rc})")

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.tam_graph_free(h)
            except Exception:
                pass
            self.handle = None

