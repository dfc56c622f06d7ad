"""Python binding of the engine's C ABI (include/rknn_gpu.h), via ctypes.

The reference's only interface is its command line (`-if <file> -k <k> -q
<index>`, rknn-inf/inf.cpp:38-119) and the counts it prints.  This module
mirrors it for Python callers and tests:

    idx = Index(fxy, uxy, fid, uid)            # rknn_index_create
    ids = idx.query(q, k)                      # one -q/-k run: sorted user ids
    res = idx.query_batch(qs, ks)              # many queries, one launch
    main(["-if", path, "-k", "5", "-q", "3"])  # the command line itself

Errors raise RkNNError carrying the library's status and message; nothing
falls back to the CPU: if the shared library or a GPU is missing, the calls
fail.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librknn_gb300.so")

MODE_FP64 = 0
MODE_FP32 = 1
_MODES = {"fp64": MODE_FP64, "fp32": MODE_FP32, MODE_FP64: MODE_FP64, MODE_FP32: MODE_FP32}

STATUS = {0: "RKNN_OK", 1: "RKNN_ERR_ARG", 2: "RKNN_ERR_OOM", 3: "RKNN_ERR_CUDA",
          4: "RKNN_ERR_TIMEOUT", 5: "RKNN_ERR_CAPACITY", 6: "RKNN_ERR_STATE"}

# every symbol include/rknn_gpu.h declares
EXPORTS = ["rknn_index_opts_default", "rknn_index_create", "rknn_index_destroy",
           "rknn_index_size", "rknn_index_get_info", "rknn_query", "rknn_query_noalloc", "rknn_query_batch", "rknn_query_batch_device",
           "rknn_batch_device_results", "rknn_sync", "rknn_set_stream", "rknn_last_stats",
           "rknn_last_zone", "rknn_set_profiling", "rknn_last_kernel_ms",
           "rknn_serve_opts_default", "rknn_serve_start", "rknn_serve_submit", "rknn_serve_wait",
           "rknn_serve_replay", "rknn_serve_stats_get", "rknn_serve_inject_fault", "rknn_serve_stop",
           "rknn_index_tune",
           "rknn_host_alloc", "rknn_host_free", "rknn_snapshot_write", "rknn_snapshot_read",
           "rknn_snapshot_free", "rknn_index_open", "rknn_index_save", "rknn_last_error", "rknn_version"]


class ServeOpts(C.Structure):
    _fields_ = [("slots", C.c_int32), ("max_batch", C.c_int32), ("scratch_bytes", C.c_int64),
                ("reserved", C.c_int32 * 8)]


class ServeStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
                ("batches", C.c_int64), ("mean_batch", C.c_double), ("max_inflight", C.c_int32),
                ("pad", C.c_int32), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("mean_ms", C.c_double), ("max_ms", C.c_double), ("throughput_qps", C.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_ if n != "pad"}


class _HostBlock:
    """Owns one rknn_host_alloc block; freed when the last array over it goes."""

    def __init__(self, nbytes: int):
        p = C.c_void_p()
        _check(load().rknn_host_alloc(int(nbytes), C.byref(p)))
        self.p = p.value

    def __del__(self):
        if self.p:
            load().rknn_host_free(C.c_void_p(self.p))
            self.p = None


def pinned_ids(n: int) -> np.ndarray:
    """An int32 array of n ids in page-locked host memory: rknn_query_batch
    copies results into it directly.  Views keep the block alive."""
    blk = _HostBlock(4 * max(1, int(n)))
    arr_t = C.c_int32 * max(1, int(n))
    cobj = arr_t.from_address(blk.p)
    cobj._owner = blk
    return np.ctypeslib.as_array(cobj)


class RkNNError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Opts(C.Structure):
    _fields_ = [("device", C.c_int32), ("fac_per_cell", C.c_float), ("usr_per_cell", C.c_float),
                ("skip_coincident", C.c_int32), ("filter", C.c_int32), ("slice_min_k", C.c_int32),
                ("users_per_thread", C.c_int32), ("verify_warps", C.c_int32), ("zone_vertex_test", C.c_int32),
                ("reserved", C.c_int32 * 1)]


class TuneResult(C.Structure):
    _fields_ = [("fac_per_cell", C.c_float), ("usr_per_cell", C.c_float),
                ("users_per_thread", C.c_int32), ("verify_warps", C.c_int32),
                ("default_ms", C.c_double), ("best_ms", C.c_double), ("trials", C.c_int32),
                ("reserved", C.c_int32 * 5)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_ if n != "reserved"}


class Info(C.Structure):
    _fields_ = [("nf", C.c_int64), ("nu", C.c_int64), ("x0", C.c_double), ("y0", C.c_double),
                ("x1", C.c_double), ("y1", C.c_double),
                ("fgrid_x0", C.c_float), ("fgrid_y0", C.c_float), ("fgrid_inv", C.c_float),
                ("fgrid_gx", C.c_int32), ("fgrid_gy", C.c_int32),
                ("ugrid_x0", C.c_float), ("ugrid_y0", C.c_float), ("ugrid_inv", C.c_float),
                ("ugrid_gx", C.c_int32), ("ugrid_gy", C.c_int32)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Stats(C.Structure):
    _fields_ = [("queries", C.c_int64), ("results", C.c_int64), ("bisectors", C.c_int64),
                ("zone_vertices_max", C.c_int64), ("zone_candidates", C.c_int64),
                ("zone_fp64", C.c_int64), ("candidates", C.c_int64), ("plane_evals", C.c_int64),
                ("survivors", C.c_int64), ("fac_checks", C.c_int64), ("rechecks", C.c_int64),
                ("overflow", C.c_int64), ("device_ms", C.c_double),
                ("zone_cycles", C.c_int64 * 8), ("zone_points", C.c_int64), ("zone_cells", C.c_int64),
                ("fused_slots", C.c_int64)]

    def as_dict(self):
        d = {n: getattr(self, n) for n, _ in self._fields_}
        d["zone_cycles"] = list(self.zone_cycles)
        return d


_lib = None


def load(path: str = LIB_PATH):
    """Load the shared library (built by rt-rknn_gb300/build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RkNNError(3, f"engine library not built: {path}")
    L = C.CDLL(path)
    vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
    L.rknn_index_opts_default.argtypes = [C.POINTER(Opts)]
    L.rknn_index_opts_default.restype = None
    L.rknn_index_create.argtypes = [vp, vp, i64, vp, vp, i64, C.POINTER(Opts), C.POINTER(vp)]
    L.rknn_index_destroy.argtypes = [vp]
    L.rknn_index_size.argtypes = [vp, C.POINTER(i64), C.POINTER(i64)]
    L.rknn_index_get_info.argtypes = [vp, C.POINTER(Info)]
    L.rknn_query.argtypes = [vp, i32, i32, i32, vp, i64, C.POINTER(i64), C.POINTER(Stats)]
    L.rknn_query_batch.argtypes = [vp, vp, vp, i32, i32, vp, i64, vp, C.POINTER(Stats)]
    L.rknn_query_noalloc.argtypes = [vp, i32, i32, i32, vp, i64, C.POINTER(i64)]
    L.rknn_host_alloc.argtypes = [i64, C.POINTER(vp)]
    L.rknn_host_free.argtypes = [vp]
    L.rknn_query_batch_device.argtypes = [vp, vp, vp, i32, i32, i32]
    L.rknn_batch_device_results.argtypes = [vp, C.POINTER(vp), C.POINTER(vp)]
    L.rknn_sync.argtypes = [vp]
    L.rknn_set_stream.argtypes = [vp, vp]
    L.rknn_last_stats.argtypes = [vp, C.POINTER(Stats)]
    L.rknn_last_zone.argtypes = [vp, i32, vp, i32, C.POINTER(i32), C.POINTER(i32)]
    L.rknn_set_profiling.argtypes = [vp, i32]
    L.rknn_last_kernel_ms.argtypes = [vp, vp]
    L.rknn_serve_opts_default.argtypes = [C.POINTER(ServeOpts)]
    L.rknn_serve_opts_default.restype = None
    L.rknn_serve_start.argtypes = [vp, C.POINTER(ServeOpts), C.POINTER(vp)]
    L.rknn_serve_submit.argtypes = [vp, i32, i32, i32, C.POINTER(C.c_uint64)]
    L.rknn_serve_wait.argtypes = [vp, C.c_uint64, i32, vp, i64, C.POINTER(i64), C.POINTER(C.c_double)]
    L.rknn_serve_replay.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp]
    L.rknn_serve_stats_get.argtypes = [vp, i32, C.POINTER(ServeStats)]
    L.rknn_serve_inject_fault.argtypes = [vp, i32, i32]
    L.rknn_serve_stop.argtypes = [vp]
    L.rknn_index_tune.argtypes = [vp, vp, vp, i32, i32, C.POINTER(TuneResult)]
    L.rknn_snapshot_write.argtypes = [C.c_char_p, vp, vp, i64, vp, vp, i64]
    L.rknn_snapshot_read.argtypes = [C.c_char_p, C.POINTER(vp), C.POINTER(vp), C.POINTER(i64), C.POINTER(vp),
                                     C.POINTER(vp), C.POINTER(i64)]
    L.rknn_snapshot_free.argtypes = [vp]
    L.rknn_snapshot_free.restype = None
    L.rknn_index_open.argtypes = [C.c_char_p, C.POINTER(Opts), C.POINTER(vp)]
    L.rknn_index_save.argtypes = [vp, C.c_char_p]
    L.rknn_last_error.restype = C.c_char_p
    L.rknn_version.restype = C.c_char_p
    for name in EXPORTS:
        fn = getattr(L, name)
        if name not in ("rknn_last_error", "rknn_version", "rknn_index_opts_default",
                        "rknn_serve_opts_default", "rknn_snapshot_free"):
            fn.restype = C.c_int
    _lib = L
    return L


_fast = None


def _fast_call():
    """The CPython entry point for rknn_query_batch (host/pycall.c, built
    beside the library where the interpreter's headers are installed), or
    False: ctypes then makes the same call."""
    global _fast
    if _fast is None:
        load()                  # the module links against the loaded library
        import importlib.util
        import sysconfig
        path = os.path.join(os.path.dirname(LIB_PATH), "_rknn_call" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))
        _fast = False
        if os.path.exists(path):
            spec = importlib.util.spec_from_file_location("_rknn_call", path)
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            _fast = mod
    return _fast


def _check(rc: int):
    if rc != 0:
        raise RkNNError(rc, load().rknn_last_error().decode())


def _ptr(a: np.ndarray):
    return a.ctypes.data if a is not None and a.size else None


def snapshot_write(path: str, fxy, fid, uxy, uid):
    """Write points as a binary index snapshot (rknn_snapshot_write)."""
    fxy = np.ascontiguousarray(fxy, dtype=np.float32).reshape(-1, 2)
    uxy = np.ascontiguousarray(uxy, dtype=np.float32).reshape(-1, 2)
    fid = np.ascontiguousarray(fid, dtype=np.int32)
    uid = np.ascontiguousarray(uid, dtype=np.int32)
    _check(load().rknn_snapshot_write(os.fsencode(path), _ptr(fxy), _ptr(fid), fxy.shape[0], _ptr(uxy),
                                      _ptr(uid), uxy.shape[0]))


def snapshot_read(path: str):
    """(fxy, fid, uxy, uid) of a binary index snapshot (rknn_snapshot_read)."""
    L = load()
    p = [C.c_void_p() for _ in range(4)]
    nf, nu = C.c_int64(), C.c_int64()
    _check(L.rknn_snapshot_read(os.fsencode(path), C.byref(p[0]), C.byref(p[1]), C.byref(nf), C.byref(p[2]),
                                C.byref(p[3]), C.byref(nu)))
    try:
        def arr(ptr, n, ct):
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ct)), shape=(n,)).copy() if n else np.zeros(0, np.dtype(ct))
        fxy = arr(p[0], 2 * nf.value, C.c_float).reshape(-1, 2)
        fid = arr(p[1], nf.value, C.c_int32)
        uxy = arr(p[2], 2 * nu.value, C.c_float).reshape(-1, 2)
        uid = arr(p[3], nu.value, C.c_int32)
    finally:
        for x in p:
            L.rknn_snapshot_free(x)
    return fxy, fid, uxy, uid


class Index:
    """Device-resident facility/user grid index (rknn_index_create)."""

    def __init__(self, fxy, uxy, fid=None, uid=None, device: int = 0,
                 fac_per_cell: float = 0.0, usr_per_cell: float = 0.0,
                 skip_coincident: bool = True, filter: str = "auto", slice_min_k: int = 0,
                 users_per_thread: int = 0, verify_warps: int = 0, zone_vertex_test: str = "reference"):
        L = load()
        self.fxy = np.ascontiguousarray(fxy, dtype=np.float32).reshape(-1, 2)
        self.uxy = np.ascontiguousarray(uxy, dtype=np.float32).reshape(-1, 2)
        nf, nu = self.fxy.shape[0], self.uxy.shape[0]
        self.fid = (np.ascontiguousarray(fid, dtype=np.int32) if fid is not None
                    else np.arange(nf, dtype=np.int32))
        self.uid = (np.ascontiguousarray(uid, dtype=np.int32) if uid is not None
                    else np.arange(nf, nf + nu, dtype=np.int32))
        o = Opts()
        L.rknn_index_opts_default(C.byref(o))
        o.device = device
        if fac_per_cell:
            o.fac_per_cell = fac_per_cell
        if usr_per_cell:
            o.usr_per_cell = usr_per_cell
        o.skip_coincident = 1 if skip_coincident else 0
        o.filter = {"auto": 0, "inf": 1, "slice": 2}[filter]
        o.slice_min_k = int(slice_min_k)
        o.users_per_thread = int(users_per_thread)
        o.verify_warps = int(verify_warps)
        o.zone_vertex_test = {"reference": 0, "boundary": 1}[zone_vertex_test]
        h = C.c_void_p()
        _check(L.rknn_index_create(_ptr(self.fxy), _ptr(self.fid), nf, _ptr(self.uxy),
                                   _ptr(self.uid), nu, C.byref(o), C.byref(h)))
        self.h = h
        self.nf, self.nu = nf, nu

    @classmethod
    def of(cls, ds, **kw):
        return cls(ds.fxy, ds.uxy, ds.fid, ds.uid, **kw)

    @classmethod
    def open(cls, path: str, **kw):
        """Index over a binary snapshot's points (the same index
        rknn_index_open builds)."""
        fxy, fid, uxy, uid = snapshot_read(path)
        return cls(fxy, uxy, fid, uid, **kw)

    def save(self, path: str):
        """Write the index's points as a binary snapshot (rknn_index_save)."""
        _check(load().rknn_index_save(self.h, os.fsencode(path)))

    def close(self):
        if getattr(self, "h", None):
            load().rknn_index_destroy(self.h)
            self.h = None
        self._flat_out = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def query(self, q: int, k: int, mode="fp64", stats: bool = False):
        """Sorted user ids of RkNN_k(q) (rknn_query: one query, one launch)."""
        L = load()
        cap = max(16, self.nu)
        out = np.empty(cap, np.int32)
        n = C.c_int64(0)
        st = Stats()
        _check(L.rknn_query(self.h, int(q), int(k), _MODES[mode], out.ctypes.data, cap,
                            C.byref(n), C.byref(st) if stats else None))
        ids = out[: n.value].copy()
        return (ids, st.as_dict()) if stats else ids

    def query_noalloc(self, q: int, k: int, mode="fp64"):
        """Sorted user ids of RkNN_k(q) through rknn_query_noalloc: no device
        allocation at query time (the scratch is a fixed device array)."""
        L = load()
        cap = max(16, self.nu)
        out = np.empty(cap, np.int32)
        n = C.c_int64(0)
        _check(L.rknn_query_noalloc(self.h, int(q), int(k), _MODES[mode], out.ctypes.data, cap,
                                    C.byref(n)))
        return out[: n.value].copy()

    def query_batch(self, qs, ks, mode="fp32", stats: bool = False):
        """List of sorted id arrays, one per query (rknn_query_batch)."""
        L = load()
        qs = np.ascontiguousarray(qs, dtype=np.int32)
        ks = np.ascontiguousarray(np.broadcast_to(np.asarray(ks, np.int32), qs.shape), dtype=np.int32)
        nq = qs.shape[0]
        off = np.zeros(nq + 1, np.int64)
        cap = getattr(self, "_cap", 1 << 16)
        st = Stats()
        while True:
            out = np.empty(max(cap, 1), np.int32)
            rc = L.rknn_query_batch(self.h, _ptr(qs), _ptr(ks), nq, _MODES[mode], out.ctypes.data,
                                    cap, off.ctypes.data, C.byref(st) if stats else None)
            if rc == 5 and off[-1] > cap:
                cap = int(off[-1])
                self._cap = cap
                continue
            _check(rc)
            break
        res = [out[off[i]:off[i + 1]].copy() for i in range(nq)]
        return (res, st.as_dict()) if stats else res

    def tune(self, qs, ks, mode="fp32") -> dict:
        """Autotune grid densities and the verification kernel's shape on a
        sample batch (rknn_index_tune); the index keeps the fastest."""
        qs = np.ascontiguousarray(qs, dtype=np.int32)
        ks = np.ascontiguousarray(np.broadcast_to(np.asarray(ks, np.int32), qs.shape), dtype=np.int32)
        r = TuneResult()
        _check(load().rknn_index_tune(self.h, _ptr(qs), _ptr(ks), qs.shape[0], _MODES[mode], C.byref(r)))
        return r.as_dict()

    def query_batch_flat(self, qs, ks, mode="fp32"):
        """(ids, offsets): the batch's results as one id array, query i's
        sorted ids at ids[offsets[i]:offsets[i+1]] (no per-query copies; the
        output buffers are reused between calls)."""
        L = load()
        fast = _fast_call()
        if type(qs) is not np.ndarray or qs.dtype != np.int32 or not qs.flags.c_contiguous:
            qs = np.ascontiguousarray(qs, dtype=np.int32)
        nq = qs.shape[0]
        if type(ks) is np.ndarray and ks.dtype == np.int32 and ks.shape == qs.shape and ks.flags.c_contiguous:
            pass
        elif np.ndim(ks) == 0:
            # a scalar k: one cached array of it per batch size
            kc = getattr(self, "_flat_k", None)
            if kc is None or kc[0] != (nq, int(ks)):
                kc = self._flat_k = ((nq, int(ks)), np.full(nq, int(ks), np.int32))
            ks = kc[1]
        else:
            ks = np.ascontiguousarray(np.broadcast_to(np.asarray(ks, np.int32), qs.shape), dtype=np.int32)
        # the offsets and the page-locked id buffer persist, their addresses
        # with them
        fo = getattr(self, "_flat_off", None)
        if fo is None or fo[0].shape[0] < nq + 1:
            a = np.zeros(max(nq + 1, 1024), np.int64)
            fo = self._flat_off = (a, a.ctypes.data)
        off, off_p = fo
        fb = getattr(self, "_flat_out", None)
        if fb is None:
            b = pinned_ids(1 << 16)
            fb = self._flat_out = (b, b.ctypes.data, b.shape[0])
        while True:
            out, out_p, cap = fb
            if fast:
                rc = fast.query_batch(self.h.value, qs, ks, _MODES[mode], out_p, cap, off_p)
            else:
                rc = L.rknn_query_batch(self.h, qs.ctypes.data, ks.ctypes.data, nq, _MODES[mode], out_p, cap,
                                        off_p, None)
            if rc == 5 and off[nq] > cap:
                b = pinned_ids(int(off[nq] * 5 // 4))
                fb = self._flat_out = (b, b.ctypes.data, b.shape[0])
                continue
            _check(rc)
            return out[: off[nq]], off[: nq + 1]

    def last_zone(self, slot: int = 0):
        """(facility indices of the bisectors in creation order, flags)."""
        L = load()
        n = C.c_int32(0)
        fl = C.c_int32(0)
        buf = np.zeros(1 << 16, np.int32)
        _check(L.rknn_last_zone(self.h, int(slot), buf.ctypes.data, buf.size, C.byref(n), C.byref(fl)))
        return buf[: min(n.value, buf.size)].copy(), fl.value

    def set_profiling(self, on: bool):
        _check(load().rknn_set_profiling(self.h, 1 if on else 0))

    def kernel_ms(self):
        """Per-kernel device ms of the last profiled call: zone (or slice
        filter), plan, verify, recount, result offsets, finalize."""
        ms = np.zeros(6, np.float64)
        _check(load().rknn_last_kernel_ms(self.h, ms.ctypes.data))
        return dict(zip(("zone", "plan", "verify", "recount", "offsets", "finalize"), ms.tolist()))

    def set_stream(self, stream_handle: int | None):
        _check(load().rknn_set_stream(self.h, C.c_void_p(stream_handle or 0)))

    def sync(self):
        _check(load().rknn_sync(self.h))

    def query_batch_device(self, d_q: int, d_k: int, nq: int, kmax: int, mode="fp32"):
        """Enqueue a batch whose q/k arrays are already on the device."""
        _check(load().rknn_query_batch_device(self.h, C.c_void_p(d_q), C.c_void_p(d_k), int(nq),
                                              int(kmax), _MODES[mode]))

    def device_results(self):
        ids, off = C.c_void_p(), C.c_void_p()
        _check(load().rknn_batch_device_results(self.h, C.byref(ids), C.byref(off)))
        return ids.value, off.value

    def info(self):
        inf = Info()
        _check(load().rknn_index_get_info(self.h, C.byref(inf)))
        return inf.as_dict()

    def last_stats(self):
        st = Stats()
        _check(load().rknn_last_stats(self.h, C.byref(st)))
        return st.as_dict()


class Server:
    """Continuous-batching server over a resident index (rknn_serve_*).

    submit() queues a request and returns a ticket; wait() returns its sorted
    ids.  Requests from any number of threads are batched as they arrive and
    run while earlier batches are still on the GPU."""

    def __init__(self, index: "Index", slots: int = 3, max_batch: int = 4096,
                 scratch_bytes: int = 256 << 20):
        L = load()
        o = ServeOpts()
        L.rknn_serve_opts_default(C.byref(o))
        o.slots, o.max_batch, o.scratch_bytes = int(slots), int(max_batch), int(scratch_bytes)
        self.index = index
        self.h = C.c_void_p()
        _check(L.rknn_serve_start(index.h, C.byref(o), C.byref(self.h)))

    def submit(self, q: int, k: int, mode="fp32") -> int:
        t = C.c_uint64(0)
        _check(load().rknn_serve_submit(self.h, int(q), int(k), _MODES[mode], C.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1, latency: bool = False):
        L = load()
        n = C.c_int64(0)
        lat = C.c_double(0)
        cap = 1024
        while True:
            out = np.empty(cap, np.int32)
            rc = L.rknn_serve_wait(self.h, C.c_uint64(ticket), int(timeout_ms), out.ctypes.data, cap,
                                   C.byref(n), C.byref(lat))
            if rc == 5 and n.value > cap:            # RKNN_ERR_CAPACITY: request kept
                cap = int(n.value)
                continue
            _check(rc)
            ids = out[: n.value].copy()
            return (ids, lat.value) if latency else ids

    def replay(self, q, k, mode, arrival_s):
        """Open-loop load: request i at arrival_s[i] s; returns (latency_ms, n_results)."""
        q = np.ascontiguousarray(q, np.int32)
        n = q.size
        k = np.ascontiguousarray(np.broadcast_to(k, n), np.int32)
        m = np.ascontiguousarray(np.broadcast_to(np.asarray([_MODES[x] for x in np.atleast_1d(mode)]), n), np.int32)
        t = np.ascontiguousarray(arrival_s, np.float64)
        lat = np.zeros(n, np.float64)
        nr = np.zeros(n, np.int64)
        _check(load().rknn_serve_replay(self.h, n, q.ctypes.data, k.ctypes.data, m.ctypes.data,
                                        t.ctypes.data, lat.ctypes.data, nr.ctypes.data))
        return lat, nr

    def inject_fault(self, kind: str, count: int = 1):
        """Failure test hook: the next `count` batches fail on the host
        ("oom": workspace allocation, RKNN_ERR_OOM; "launch": after the
        input copy, RKNN_ERR_CUDA)."""
        _check(load().rknn_serve_inject_fault(self.h, {"oom": 1, "launch": 2}[kind], int(count)))

    def stats(self, reset: bool = False) -> dict:
        st = ServeStats()
        _check(load().rknn_serve_stats_get(self.h, 1 if reset else 0, C.byref(st)))
        return st.as_dict()

    def stop(self):
        if self.h:
            load().rknn_serve_stop(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.stop()

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass


def main(argv=None) -> int:
    """The reference's command line (`-if <file> -k <k> -q <index>`), with the
    result set written to log/<mode>_k<k>_q<q>.txt."""
    import argparse
    import time
    sys.path.insert(0, HERE)
    import datagen
    p = argparse.ArgumentParser(prog="rknn")
    p.add_argument("-if", "--infile", dest="infile", required=True)
    p.add_argument("-k", type=int, default=4)
    p.add_argument("-q", type=int, default=0)
    p.add_argument("-al", "--algorithm", default="all")
    p.add_argument("--mode", default="fp64", choices=["fp64", "fp32"])
    p.add_argument("--filter", default="inf", choices=["inf", "slice", "auto"])
    p.add_argument("--log", default="log")
    a = p.parse_args(argv)
    if a.k <= 0:
        print(f"Invalid value for k: {a.k}. It must be a positive integer.", file=sys.stderr)
        return 1
    print("Loading data...")
    ds = datagen.read_text(a.infile)
    print(f"Loaded {ds.nf} facilities and {ds.nu} users.")
    t0 = time.time()
    with Index.of(ds, filter=a.filter) as idx:
        print(f"Grid index is built in {time.time() - t0:g}[s].\n")
        t0 = time.time()
        ids, st = idx.query(a.q, a.k, a.mode, stats=True)
        print(f"Total bisectors created: {st['bisectors']}")
        print(f"Found {len(ids)} RkNN results.")
        print(f"Total time: {time.time() - t0:g}[s].\n")
    os.makedirs(a.log, exist_ok=True)
    with open(os.path.join(a.log, f"{a.mode}_k{a.k}_q{a.q}.txt"), "w") as fh:
        fh.writelines(f"{int(i)}\n" for i in ids)
    return 0


if __name__ == "__main__":
    sys.exit(main())
