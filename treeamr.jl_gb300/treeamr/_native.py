"""ctypes binding of libtreeamr_cuda.so and the schedule flattening.

The C ABI is declared in ``include/treeamr_cuda.h``.  ``Descriptor`` turns a
``GhostSchedule`` into the struct-of-arrays ``tam_schedule_desc`` (what the
Julia host would hand the library from ``src/schedule.jl``).  ``build()``
compiles the library for sm_103a in-tree; ``lib()`` loads it and raises if it
is missing -- there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor
from typing import List, Optional

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT_DIR = os.path.dirname(os.path.dirname(PKG_DIR))          # the repository
CSRC_DIR = os.path.join(os.path.dirname(PKG_DIR), "csrc")
INCLUDE_DIR = os.path.join(ROOT_DIR, "include")
BUILD_DIR = os.path.join(CSRC_DIR, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libtreeamr_cuda.so")

ABI_VERSION = 2
TAM_F32, TAM_F64 = 1, 2
TAM_OK, TAM_EINVAL, TAM_EUNSUPPORTED = 0, -1, -6
TAM_STAGE_ALL_FIRST, TAM_STAGE_ALL_LAST = -1, 0x7FFFFFFF
TAM_METHOD_FUSED, TAM_METHOD_PLAIN = 0, 1

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = ["tam_fused_f64_d3.cu", "tam_fused_f64_d2.cu", "tam_fused_f64_d1.cu",
           "tam_fused_f32.cu", "tam_kernels.cu", "tam_api.cpp",
           "tam_adjoint.cu", "tam_batch.cpp", "tam_wave.cu", "tam_state.cu", "tam_boundary.cu",
           "tam_runtime.cpp"]


class tam_stencil(C.Structure):
    _fields_ = [("targetfirst", C.c_int32), ("ntarget", C.c_int32), ("order", C.c_int32),
                ("unit", C.c_int32), ("srcstart", C.c_int64), ("weights", C.c_int64)]


class tam_group(C.Structure):
    _fields_ = [("kind", C.c_int32), ("stage", C.c_int32), ("factorcol", C.c_int32),
                ("bounded", C.c_int32), ("orientation", C.c_int32), ("axes", C.c_int32),
                ("first", C.c_int64), ("ntransfers", C.c_int64),
                ("stencil", tam_stencil * 3)]


class tam_schedule_desc(C.Structure):
    _fields_ = [("abi_version", C.c_int32), ("ndim", C.c_int32), ("dtype", C.c_int32),
                ("stored", C.c_int32 * 3), ("nblocks", C.c_int64), ("ngroups", C.c_int32),
                ("nfactorcols", C.c_int32), ("groups", C.POINTER(tam_group)),
                ("ntransfers", C.c_int64), ("targetblocks", C.POINTER(C.c_int32)),
                ("sourceblocks", C.POINTER(C.c_int32)), ("nsrcstart", C.c_int64),
                ("srcstart", C.POINTER(C.c_int32)), ("nweights", C.c_int64),
                ("weights", C.c_void_p)]


TAM_BC_CONSTANT, TAM_BC_POLYNOMIAL, TAM_BC_MAX_TERMS = 1, 2, 20


class tam_boundary_region(C.Structure):
    _fields_ = [("block", C.c_int32), ("first", C.c_int32 * 3), ("n", C.c_int32 * 3),
                ("ghosts", C.c_int32 * 3), ("stagger", C.c_int32 * 3), ("clamps", C.c_int32 * 3),
                ("pad", C.c_int32),
                ("base", C.c_int64 * 3), ("lo", C.c_double * 3), ("h", C.c_double)]


class tam_boundary_fn(C.Structure):
    _fields_ = [("kind", C.c_int32), ("nterms", C.c_int32), ("relative", C.c_int32),
                ("exps", (C.c_int32 * 3) * TAM_BC_MAX_TERMS)]


class tam_state_layout(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("ndim", C.c_int32), ("own", C.c_int32 * 3),
                ("stored", C.c_int32 * 3), ("ghosts", C.c_int32 * 3), ("nvars", C.c_int32),
                ("nblocks", C.c_int64)]


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class Descriptor:
    """The flattened schedule: pools of srcstarts and weights, the
    concatenated block lists and one ``tam_group`` per TransferGroup, in the
    order the fill runs the stages.  Keeps its arrays alive."""

    def __init__(self, schedule, groups=None):
        from .schedule import KINDCODE
        groups = schedule.all_groups() if groups is None else groups
        D = schedule.forest.D
        T = np.dtype(schedule.T)
        ss_pool: List[np.ndarray] = []
        w_pool: List[np.ndarray] = []
        tb_list, sb_list = [], []
        nss = nw = ntr = 0
        self.groups_arr = (tam_group * max(1, len(groups)))()
        memo = {}
        for gi, g in enumerate(groups):
            cg = self.groups_arr[gi]
            cg.kind = KINDCODE[g.kind]
            cg.stage = g.stage
            cg.factorcol = g.factorcol
            cg.bounded = getattr(g, "bounded", 0)
            cg.orientation = getattr(g, "orientation", 0)
            cg.axes = 0
            if cg.orientation:
                for e, (p, f) in enumerate(zip(g.perm, g.flip)):
                    cg.axes |= (int(p) << (2 * e)) | (int(bool(f)) << (8 + e))
            cg.first = ntr
            cg.ntransfers = g.ntransfers()
            tb_list.append(g.targetblocks)
            sb_list.append(g.sourceblocks)
            ntr += g.ntransfers()
            for d in range(3):
                st = cg.stencil[d]
                if d >= D:
                    st.targetfirst, st.ntarget, st.order, st.unit = 1, 1, 1, 1
                    st.srcstart, st.weights = 0, 0
                    continue
                s = g.stencils[d]
                key = id(s)
                if key not in memo:
                    memo[key] = (nss, nw)
                    ss_pool.append(s.srcstart)
                    w_pool.append(np.asfortranarray(s.weights).ravel(order="F"))
                    nss += s.ntarget
                    nw += s.order * s.ntarget
                st.targetfirst, st.ntarget, st.order = s.targetfirst, s.ntarget, s.order
                st.unit = 1 if s.unit else 0
                st.srcstart, st.weights = memo[key]
        self.srcstart = np.ascontiguousarray(np.concatenate(ss_pool) if ss_pool else
                                             np.zeros(1, np.int32), dtype=np.int32)
        self.weights = np.ascontiguousarray(np.concatenate(w_pool) if w_pool else
                                            np.zeros(1, T), dtype=T)
        self.targetblocks = np.ascontiguousarray(np.concatenate(tb_list) if tb_list else
                                                 np.zeros(1, np.int32), dtype=np.int32)
        self.sourceblocks = np.ascontiguousarray(np.concatenate(sb_list) if sb_list else
                                                 np.zeros(1, np.int32), dtype=np.int32)
        d = tam_schedule_desc()
        d.abi_version = ABI_VERSION
        d.ndim = D
        d.dtype = TAM_F64 if T == np.float64 else TAM_F32
        for k in range(3):
            d.stored[k] = schedule.stored[k] if k < D else 1
        d.nblocks = schedule.forest.nleaves()
        d.ngroups = len(groups)
        seam = getattr(schedule.forest, "hasrotating", None)
        d.nfactorcols = 3 ** D * (4 if seam is not None and seam() else 1)
        d.groups = C.cast(self.groups_arr, C.POINTER(tam_group))
        d.ntransfers = ntr
        d.targetblocks = _ptr(self.targetblocks, C.c_int32)
        d.sourceblocks = _ptr(self.sourceblocks, C.c_int32)
        d.nsrcstart = nss
        d.srcstart = _ptr(self.srcstart, C.c_int32)
        d.nweights = nw
        d.weights = self.weights.ctypes.data
        self.desc = d
        self.dtype = T
        self.ndim = D

    def ref(self):
        return C.byref(self.desc)


# --- build --------------------------------------------------------------------

_build_lock = threading.Lock()


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libtreeamr_cuda.so for sm_103a into ``csrc/_build``."""
    with _build_lock:
        os.makedirs(BUILD_DIR, exist_ok=True)
        srcs = [os.path.join(CSRC_DIR, s) for s in SOURCES]
        hdrs = [os.path.join(CSRC_DIR, "tam_internal.h"), os.path.join(CSRC_DIR, "tam_kernels.cuh"),
                os.path.join(INCLUDE_DIR, "treeamr_cuda.h")]
        newest = max(os.path.getmtime(p) for p in srcs + hdrs + [__file__])
        if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
            return LIB_PATH
        nvcc = _nvcc()
        common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                  "-I", INCLUDE_DIR, "-I", CSRC_DIR] + ARCH_FLAGS

        def compile_one(src):
            obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
            cmd = [nvcc] + common + ["-c", src, "-o", obj]
            if src.endswith(".cpp"):
                cmd = [nvcc, "-x", "cu"] + common + ["-c", src, "-o", obj]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
            if verbose and r.stderr:
                print(r.stderr)
            return obj

        with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
            objs = list(ex.map(compile_one, srcs))
        tmp = LIB_PATH + ".tmp"
        # the shared CUDA runtime: the one the host process (torch) has loaded,
        # so page-locked buffers it allocated are known to the library's copies
        cmd = [nvcc, "-shared", "-cudart", "shared"] + ARCH_FLAGS + objs + ["-o", tmp]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
        return LIB_PATH


# --- load ---------------------------------------------------------------------

_lib: Optional[C.CDLL] = None


def _declare(lib: C.CDLL):
    vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
    lib.tam_abi_version.restype = C.c_int
    lib.tam_init.argtypes = [C.c_int, C.POINTER(vp)]
    lib.tam_free.argtypes = [vp]
    lib.tam_free.restype = None
    lib.tam_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    lib.tam_schedule_upload.argtypes = [vp, C.POINTER(tam_schedule_desc), C.POINTER(vp)]
    lib.tam_schedule_free.argtypes = [vp]
    lib.tam_schedule_free.restype = None
    lib.tam_schedule_info.argtypes = [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64),
                                      C.POINTER(i32)]
    lib.tam_schedule_stage_groups.argtypes = [vp, C.POINTER(i32), C.POINTER(i32)]
    lib.tam_schedule_stage_groups.restype = C.c_int
    for name in ("tam_fill", "tam_fill_plain", "tam_fill_adjoint", "tam_fill_adjoint_static"):
        if not hasattr(lib, name):
            continue
        f = getattr(lib, name)
        f.argtypes = [vp, vp, i32, i64, vp, i32, i32, vp]
        f.restype = C.c_int
    lib.tam_axis_project.argtypes = [i32, vp, i64, i32, vp, i32, i64, vp, i32, vp, vp, vp]
    lib.tam_axis_project.restype = C.c_int
    lib.tam_autotune.argtypes = [vp, vp, i32, i64, vp, i32, vp, C.POINTER(i64), C.POINTER(i64),
                                 C.POINTER(i64), C.POINTER(C.c_double)]
    lib.tam_autotune.restype = C.c_int
    lib.tam_graph_capture_rk4.argtypes = [vp, i32, vp, i32, i32, vp, vp, vp, vp, i64, i32, vp,
                                          i64, C.c_double, i32, i32, C.POINTER(vp)]
    lib.tam_graph_capture_rk4.restype = C.c_int
    lib.tam_graph_launch.argtypes = [vp, vp]
    lib.tam_graph_launch.restype = C.c_int
    lib.tam_graph_free.argtypes = [vp]
    lib.tam_graph_free.restype = None
    lib.tam_fill_host_own.argtypes = [vp, C.POINTER(tam_state_layout), vp, vp, vp, i32, i64,
                                      vp, i32, i32, vp]
    lib.tam_fill_host_own.restype = C.c_int
    lib.tam_fill_ex.argtypes = [vp, vp, vp, i32, i64, vp, vp, i32, i32, i32, vp]
    lib.tam_fill_ex.restype = C.c_int
    lib.tam_fill_adjoint_ex.argtypes = [vp, vp, i32, i64, vp, vp, i32, i32, vp, C.c_size_t,
                                        vp]
    lib.tam_fill_adjoint_ex.restype = C.c_int
    lib.tam_fill_adjoint_alt.argtypes = [vp, vp, vp, i32, i64, vp, vp, i32, i32, vp,
                                         C.c_size_t, vp]
    lib.tam_fill_adjoint_alt.restype = C.c_int
    lib.tam_regrid_upload.argtypes = [vp, C.POINTER(tam_schedule_desc), i64, C.POINTER(vp)]
    lib.tam_regrid_upload.restype = C.c_int
    lib.tam_regrid_transfer.argtypes = [vp, vp, i64, vp, i64, i32, vp]
    lib.tam_regrid_transfer.restype = C.c_int
    lib.tam_boundary_apply.argtypes = [i32, vp, i32, tam_boundary_fn, vp, vp, i32,
                                       C.POINTER(C.c_int32), vp]
    lib.tam_boundary_apply.restype = C.c_int
    lib.tam_scatter.argtypes = [C.POINTER(tam_state_layout), vp, vp, vp]
    lib.tam_scatter.restype = C.c_int
    lib.tam_gather.argtypes = [C.POINTER(tam_state_layout), vp, vp, vp]
    lib.tam_gather.restype = C.c_int
    lib.tam_fill_host.argtypes = [vp, vp, vp, vp, i32, i64, vp, i32, i32, vp]
    lib.tam_fill_host.restype = C.c_int
    lib.tam_device_status.argtypes = [vp, vp, C.POINTER(i32)]
    lib.tam_selftest.argtypes = [vp, i32, i64, C.c_uint64, C.POINTER(i64)]
    lib.tam_adjoint_scratch_bytes.argtypes = [vp, i32, C.POINTER(C.c_size_t)]
    lib.tam_adjoint_scratch_bytes.restype = C.c_int
    lib.tam_fill_adjoint_scratch.argtypes = [vp, vp, i32, i64, vp, i32, i32, vp, C.c_size_t, vp]
    lib.tam_fill_adjoint_scratch.restype = C.c_int
    lib.tam_batch_create.argtypes = [vp, C.POINTER(vp), i32, C.POINTER(i64), C.POINTER(i64),
                                     C.POINTER(vp)]
    lib.tam_batch_create.restype = C.c_int
    lib.tam_batch_free.argtypes = [vp]
    lib.tam_batch_free.restype = None
    for name in ("tam_batch_fill", "tam_batch_fill_adjoint"):
        f = getattr(lib, name)
        f.argtypes = [vp, vp, i64, i32, vp, i64, i32, i32, vp]
        f.restype = C.c_int
    for name in ("tam_batch_fill_ex", "tam_batch_fill_adjoint_ex"):
        f = getattr(lib, name)
        f.argtypes = [vp, vp, i64, i32, vp, i64, vp, i32, i32, vp]
        f.restype = C.c_int
    lib.tam_batch_device_status.argtypes = [vp, vp, C.POINTER(i32)]
    lib.tam_batch_device_status.restype = C.c_int
    lib.tam_batch_set_option.argtypes = [vp, i32, i64]
    lib.tam_batch_set_option.restype = C.c_int
    lib.tam_schedule_set_option.argtypes = [vp, i32, i64]
    lib.tam_schedule_get_option.argtypes = [vp, i32, C.POINTER(i64)]
    for name in ("tam_init", "tam_last_error", "tam_schedule_upload", "tam_schedule_info",
                 "tam_device_status", "tam_selftest", "tam_schedule_set_option",
                 "tam_schedule_get_option"):
        getattr(lib, name).restype = C.c_int


def lib() -> C.CDLL:
    """The loaded library.  Raises if it was not built: the engine has no
    CPU or library fallback."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"libtreeamr_cuda.so is not built ({LIB_PATH}); run treeamr._native.build() "
                "(or __graft_entry__.build()) first")
        l = C.CDLL(LIB_PATH)
        _declare(l)
        if l.tam_abi_version() != ABI_VERSION:
            raise RuntimeError("libtreeamr_cuda.so has a different ABI version")
        _lib = l
    return _lib


class TamError(RuntimeError):
    pass


def last_error(ctx) -> str:
    buf = C.create_string_buffer(1024)
    lib().tam_last_error(ctx, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, ctx, what: str):
    if rc != 0:
        raise TamError(f"{what} failed ({rc}): {last_error(ctx)}")


_contexts = {}


def context(device: int):
    """One library context per CUDA device, opened on first use."""
    if device not in _contexts:
        ctx = C.c_void_p()
        check(lib().tam_init(device, C.byref(ctx)), None, "tam_init")
        _contexts[device] = ctx
    return _contexts[device]
