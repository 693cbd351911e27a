"""Batched layouts: many independent jobs advanced by one launch per tick.

`Batch` wraps the cgl_batch_* C ABI.  Each job is equivalent to a plain
engine created with the same config, given the same positions and links,
rendered and started at alpha 1; it advances on every `step` until its tick
budget is spent or (optionally) alpha falls below ALPHA_MIN.
"""
import ctypes as C

import numpy as np

from . import _abi
from ._calls import StatusError, _f32, _fptr
from .engine import load_library


def _declare(lib):
    if getattr(lib, "_batch_declared", False):
        return
    B = C.c_void_p
    f = C.POINTER(C.c_float)
    lib.cgl_batch_create.argtypes = [C.c_int32, C.c_double, C.POINTER(C.c_void_p)]
    lib.cgl_batch_destroy.argtypes = [B]
    lib.cgl_batch_add.argtypes = [B, C.POINTER(_abi.Config), f, C.c_uint64, f, C.c_uint64, C.c_uint32, C.c_int32,
                                  C.POINTER(C.c_uint32)]
    lib.cgl_batch_add_many.argtypes = [B, C.c_uint32, C.POINTER(_abi.BatchJob), C.POINTER(C.c_uint32), C.c_uint32,
                                       C.POINTER(C.c_uint32)]
    lib.cgl_batch_get_positions_many.argtypes = [B, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_void_p),
                                                 C.POINTER(C.c_uint64)]
    lib.cgl_batch_remove.argtypes = [B, C.c_uint32]
    lib.cgl_batch_step.argtypes = [B, C.c_uint32]
    lib.cgl_batch_synchronize.argtypes = [B]
    lib.cgl_batch_get_point_positions.argtypes = [B, C.c_uint32, f, C.c_uint64]
    lib.cgl_batch_get_state.argtypes = [B, C.c_uint32, C.POINTER(_abi.State)]
    lib.cgl_batch_get_info.argtypes = [B, C.POINTER(_abi.BatchInfo)]
    lib.cgl_batch_last_error.argtypes = [B]
    lib.cgl_batch_last_error.restype = C.c_char_p
    for fn in ("create", "destroy", "add", "add_many", "remove", "step", "synchronize", "get_point_positions",
               "get_positions_many", "get_state", "get_info"):
        getattr(lib, "cgl_batch_" + fn).restype = C.c_int
    lib._batch_declared = True


class Batch:
    def __init__(self, device=0, hbm_budget_bytes=0.0):
        self._lib = load_library()
        _declare(self._lib)
        h = C.c_void_p()
        st = self._lib.cgl_batch_create(int(device), float(hbm_budget_bytes), C.byref(h))
        if st != _abi.CGL_OK:
            raise StatusError("cgl_batch_create", st, "(no usable CUDA device?)")
        self._h = h
        self._n = {}

    def _check(self, name, st):
        if st not in (_abi.CGL_OK, _abi.CGL_WARNING):
            t = self._lib.cgl_batch_last_error(self._h)
            raise StatusError("cgl_batch_" + name, st, t.decode() if t else "")
        return st

    def add(self, positions, links=None, max_ticks=0, stop_below_alpha_min=False, cfg=None, sizes=None, **fields):
        """Add one job; `sizes` are its per-point sizes (the collision radii, Graph.setPointSizes)."""
        if sizes is not None:
            return self.add_many([dict(positions=positions, links=links, max_ticks=max_ticks,
                                       stop_below_alpha_min=stop_below_alpha_min, cfg=cfg, sizes=sizes, **fields)])[0]
        if cfg is None:
            cfg = _abi.make_config(**fields)
        xy = _f32(positions)
        ln = _f32(links) if links is not None else np.zeros(0, dtype=np.float32)
        gid = C.c_uint32()
        self._check("add", self._lib.cgl_batch_add(self._h, C.byref(cfg), _fptr(xy), xy.size, _fptr(ln), ln.size,
                                                   int(max_ticks), int(bool(stop_below_alpha_min)), C.byref(gid)))
        self._n[gid.value] = xy.size // 2
        return gid.value

    def add_many(self, jobs, threads=0, until_full=False):
        """Add jobs (dicts of add()'s arguments) with their host work on `threads` host threads
        (0 = one per core); returns their ids in order.  until_full: a job refused for device
        memory (CGL_OOM) ends the call without an error, and the ids of the jobs added before it
        are returned."""
        keep = []
        arr = (_abi.BatchJob * len(jobs))()
        for k, jb in enumerate(jobs):
            jb = dict(jb)
            cfg = jb.pop("cfg", None)
            pos = _f32(jb.pop("positions"))
            links = jb.pop("links", None)
            ln = _f32(links) if links is not None else np.zeros(0, dtype=np.float32)
            sizes = jb.pop("sizes", None)
            sz = _f32(sizes) if sizes is not None else None
            max_ticks = jb.pop("max_ticks", 0)
            stop = jb.pop("stop_below_alpha_min", False)
            if cfg is None:
                cfg = _abi.make_config(**jb)
            keep += [cfg, pos, ln, sz]
            arr[k].cfg = C.pointer(cfg)
            arr[k].xy = _fptr(pos)
            arr[k].n_floats = pos.size
            arr[k].links = _fptr(ln)
            arr[k].n_link_floats = ln.size
            if sz is not None:
                arr[k].sizes = _fptr(sz)
                arr[k].n_sizes = sz.size
            arr[k].max_ticks = int(max_ticks)
            arr[k].stop_below_alpha_min = int(bool(stop))
        ids = (C.c_uint32 * len(jobs))()
        added = C.c_uint32()
        st = self._lib.cgl_batch_add_many(self._h, len(jobs), arr, ids, int(threads), C.byref(added))
        for k in range(added.value):
            self._n[ids[k]] = int(arr[k].n_floats) // 2
        if until_full and st == _abi.CGL_OOM:
            return [ids[k] for k in range(added.value)]
        self._check("add_many", st)
        return [ids[k] for k in range(len(jobs))]

    def remove(self, job):
        self._check("remove", self._lib.cgl_batch_remove(self._h, int(job)))
        self._n.pop(job, None)

    def step(self, ticks=1):
        return self._check("step", self._lib.cgl_batch_step(self._h, int(ticks)))

    def synchronize(self):
        return self._check("synchronize", self._lib.cgl_batch_synchronize(self._h))

    def get_point_positions(self, job):
        out = np.empty(2 * self._n[job], dtype=np.float32)
        self._check("get_point_positions", self._lib.cgl_batch_get_point_positions(self._h, int(job), _fptr(out),
                                                                                   out.size))
        return out

    def get_positions_many(self, jobs):
        """Positions of several jobs with one device-to-host copy; a list of arrays in job order."""
        jobs = list(jobs)
        outs = [np.empty(2 * self._n[j], dtype=np.float32) for j in jobs]
        ids = (C.c_uint32 * len(jobs))(*jobs)
        ptrs = (C.c_void_p * len(jobs))(*[o.ctypes.data for o in outs])
        caps = (C.c_uint64 * len(jobs))(*[o.size for o in outs])
        self._check("get_positions_many", self._lib.cgl_batch_get_positions_many(self._h, len(jobs), ids, ptrs, caps))
        return outs

    def state(self, job):
        s = _abi.State()
        self._check("get_state", self._lib.cgl_batch_get_state(self._h, int(job), C.byref(s)))
        return s

    def info(self):
        i = _abi.BatchInfo()
        self._check("get_info", self._lib.cgl_batch_get_info(self._h, C.byref(i)))
        return i

    def close(self):
        if self._h:
            self._lib.cgl_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
