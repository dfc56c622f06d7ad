"""ctypes wrapper of the exact CPU oracle (oracle/rknn_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check in
__graft_entry__.py and by bench.py's CPU-baseline leg, never by the engine.

`Oracle(ds).query(q, k)` returns the sorted user ids of RkNN_k(q) under the
strict-< rule (rknn-inf/inf.h:77-93); `tie="naive"` reproduces rknn-naive's
(distance, x, y, id) ordering (rknn-naive/rknn.cpp:53-57,176-185) for
integer-coordinate data.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "librknn_oracle.so")


def build(force: bool = False) -> str:
    """Compile the oracle shared library (plain C, gcc)."""
    src = os.path.join(HERE, "rknn_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE, "librknn_oracle.so"])
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.orc_build.restype = C.c_void_p
        L.orc_build.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p]
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_query.restype = C.c_int
        L.orc_query.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                C.c_void_p, C.POINTER(C.c_int64)]
        L.orc_count_closer.restype = C.c_int
        L.orc_count_closer.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int32]
        L.orc_query_brute.restype = C.c_int
        L.orc_query_brute.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                      C.c_int64, C.c_int32, C.c_void_p]
        L.orc_query_many.restype = C.c_void_p
        L.orc_query_many.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32]
        L.orc_many_pairs.restype = C.c_int64
        L.orc_many_pairs.argtypes = [C.c_void_p]
        L.orc_many_fetch.restype = C.c_int
        L.orc_many_fetch.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_many_free.argtypes = [C.c_void_p]
        for name in ("orc_sign_d2diff", "orc_sign_d2diff_expansion"):
            fn = getattr(L, name)
            fn.restype = C.c_int
            fn.argtypes = [C.c_float] * 6
        _lib = L
    return _lib


def sign_d2diff(u, f, q, expansion_only: bool = False) -> int:
    """Exact sign of d2(u,f) - d2(u,q) for float32 points."""
    fn = lib().orc_sign_d2diff_expansion if expansion_only else lib().orc_sign_d2diff
    return int(fn(*(float(np.float32(v)) for v in (*u, *f, *q))))


class Oracle:
    def __init__(self, fxy, uxy, fid=None, uid=None):
        self.fxy = np.ascontiguousarray(fxy, dtype=np.float32)
        self.uxy = np.ascontiguousarray(uxy, dtype=np.float32)
        nf, nu = self.fxy.shape[0], self.uxy.shape[0]
        self.fid = (np.ascontiguousarray(fid, dtype=np.int32) if fid is not None
                    else np.arange(nf, dtype=np.int32))
        # default ids as the engine's: facilities 0..nf-1, users nf..nf+nu-1
        self.uid = (np.asarray(uid, dtype=np.int64) if uid is not None
                    else np.arange(nf, nf + nu, dtype=np.int64))
        self.h = lib().orc_build(self.fxy.ctypes.data, nf, self.uxy.ctypes.data, nu,
                                 self.fid.ctypes.data)
        if not self.h:
            raise MemoryError("oracle index build failed")
        self.nthreads = os.cpu_count() or 1

    @classmethod
    def of(cls, ds):
        return cls(ds.fxy, ds.uxy, ds.fid, ds.uid)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().orc_free(h)
            self.h = None

    def flags(self, q: int, k: int, tie: str = "strict") -> np.ndarray:
        out = np.zeros(self.uxy.shape[0], np.uint8)
        n = C.c_int64(0)
        rc = lib().orc_query(self.h, int(q), int(k), 0 if tie == "strict" else 1,
                             self.nthreads, out.ctypes.data, C.byref(n))
        if rc != 0:
            raise ValueError(f"oracle query rejected (q={q}, k={k})")
        return out

    def query(self, q: int, k: int, tie: str = "strict") -> np.ndarray:
        """Sorted user ids of RkNN_k(q)."""
        f = self.flags(q, k, tie)
        return np.sort(self.uid[np.nonzero(f)[0]])

    def query_many(self, qs, ks):
        """All queries (qs[s], ks[s]) at once, evaluated user by user
        (orc_query_many): (offsets[nq+1], ids) with the sorted result ids of
        slot s in ids[offsets[s]:offsets[s+1]]."""
        qs = np.ascontiguousarray(qs, dtype=np.int64)
        ks = np.ascontiguousarray(np.broadcast_to(np.asarray(ks, np.int32), qs.shape), dtype=np.int32)
        L = lib()
        r = L.orc_query_many(self.h, qs.ctypes.data, ks.ctypes.data, qs.shape[0], self.nthreads)
        if not r:
            raise ValueError("oracle batch rejected (bad query or out of memory)")
        try:
            n = int(L.orc_many_pairs(r))
            off = np.zeros(qs.shape[0] + 1, np.int64)
            users = np.zeros(max(n, 1), np.int32)
            if L.orc_many_fetch(r, off.ctypes.data, users.ctypes.data) != 0:
                raise ValueError("oracle batch fetch failed")
        finally:
            L.orc_many_free(r)
        ids = self.uid[users[:n]]
        if not np.all(np.diff(self.uid) > 0):
            # users come out in input order: sort each slot's ids
            slot = np.repeat(np.arange(qs.shape[0]), np.diff(off))
            ids = ids[np.lexsort((ids, slot))]
        return off, ids

    def count_closer(self, u: int, q: int, cap: int = 1 << 30) -> int:
        return int(lib().orc_count_closer(self.h, int(u), int(q), int(cap)))


def brute_flags(fxy, uxy, q, k) -> np.ndarray:
    fxy = np.ascontiguousarray(fxy, dtype=np.float32)
    uxy = np.ascontiguousarray(uxy, dtype=np.float32)
    out = np.zeros(uxy.shape[0], np.uint8)
    rc = lib().orc_query_brute(fxy.ctypes.data, fxy.shape[0], uxy.ctypes.data,
                               uxy.shape[0], int(q), int(k), out.ctypes.data)
    if rc != 0:
        raise ValueError("bad query")
    return out


# ------------------------------------------------------------------ inf port
PORT = os.path.join(HERE, "inf_port.so")
_port = None


def port_lib():
    """The C restatement of rknn-inf's query path (oracle/inf_port.c)."""
    global _port
    if _port is None:
        src = os.path.join(HERE, "inf_port.c")
        if not os.path.exists(PORT) or os.path.getmtime(PORT) < os.path.getmtime(src):
            subprocess.check_call(["make", "-s", "-C", HERE, "inf_port.so"])
        L = C.CDLL(PORT)
        L.ip_build.restype = C.c_void_p
        L.ip_build.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int,
                               C.c_float, C.c_float, C.c_float, C.c_int, C.c_int]
        L.ip_free.argtypes = [C.c_void_p]
        L.ip_query.restype = C.c_int
        L.ip_query.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_void_p,
                               C.c_int32, C.c_void_p, C.c_void_p]
        L.ip_query_many.restype = C.c_int
        L.ip_query_many.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                    C.c_void_p]
        _port = L
    return _port


class InfPort:
    """rknn-inf's filter + verification on the CPU.  grid=None: R-tree
    (timing baseline); grid=(x0, y0, inv, gx, gy): the engine's facility grid
    (bisector-set audit of the GPU zone kernel)."""

    def __init__(self, fxy, uxy, grid=None, uid=None):
        self.fxy = np.ascontiguousarray(fxy, dtype=np.float32)
        self.uxy = np.ascontiguousarray(uxy, dtype=np.float32)
        nu = self.uxy.shape[0]
        self.uid = (np.asarray(uid, np.int64) if uid is not None else
                    np.arange(self.fxy.shape[0], self.fxy.shape[0] + nu))
        g = grid or (0.0, 0.0, 0.0, 0, 0)
        self.h = port_lib().ip_build(self.fxy.ctypes.data, self.fxy.shape[0], self.uxy.ctypes.data,
                                     nu, 1 if grid else 0, *g)
        if not self.h:
            raise MemoryError("port index build failed")

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            port_lib().ip_free(h)
            self.h = None

    def query(self, q, k, skip_coincident=True, verify=True):
        """(bisector facility indices in creation order, result ids or None, stats)."""
        bis = np.zeros(1 << 16, np.int32)
        flags = np.zeros(self.uxy.shape[0], np.uint8) if verify else None
        st = np.zeros(5, np.int64)
        rc = port_lib().ip_query(self.h, int(q), int(k), 1 if skip_coincident else 0,
                                 bis.ctypes.data, bis.size,
                                 flags.ctypes.data if verify else None, st.ctypes.data)
        if rc:
            raise ValueError("port query rejected")
        ids = np.sort(self.uid[np.nonzero(flags)[0]]) if verify else None
        return bis[: min(int(st[0]), bis.size)].copy(), ids, \
            dict(bisectors=int(st[0]), vmax=int(st[1]), pts=int(st[2]), nodes=int(st[3]))

    def query_many(self, qs, ks, nthreads=None):
        qs = np.ascontiguousarray(qs, np.int64)
        ks = np.ascontiguousarray(np.broadcast_to(np.asarray(ks, np.int32), qs.shape), np.int32)
        cnt = np.zeros(qs.shape[0], np.int64)
        rc = port_lib().ip_query_many(self.h, qs.ctypes.data, ks.ctypes.data, qs.shape[0],
                                      nthreads or os.cpu_count() or 1, cnt.ctypes.data)
        if rc:
            raise ValueError("port batch failed")
        return cnt
