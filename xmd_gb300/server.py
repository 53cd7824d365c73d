"""Continuous-batching serving loop (xmd_gpu_server_* of include/xmd_gpu.h).

A worker thread inside the library owns one engine context: requests are
admitted into replica slots while the capacity reserved from the HBM budget
has room, advance together in batched launches, and leave as soon as their
steps are done.  There is no counterpart in the reference, whose driver runs
one system per process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import check, dptr, iptr, u8ptr


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32)) if a is not None and len(a) else None


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None and len(a) else None


class Server:
    def __init__(self, yaml: str = "", hbm_budget: int = 4 << 30, max_beads: int = 200_000,
                 chunk_steps: int = 256):
        self.lib = abi.load()
        h = C.c_void_p()
        check(self.lib.xmd_gpu_server_create(yaml.encode(), int(hbm_budget), int(max_beads), int(chunk_steps),
                                             C.byref(h)))
        self.h = h
        self.sizes = {}

    def close(self):
        if self.h:
            self.lib.xmd_gpu_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, s, nsteps: int, temperature: float | None = None, seed: int | None = None) -> int:
        """Queue a synth.System (or anything with its fields) for `nsteps`
        steps; the arrays are copied before this returns."""
        keep = []

        def arr(x, dt):
            a = np.ascontiguousarray(x, dtype=dt)
            keep.append(a)
            return a
        q = abi.Request()
        q.n = s.n
        q.chain_idx = iptr(arr(s.chain, np.int32))
        q.seq_idx = iptr(arr(s.seq, np.int32))
        q.atype = u8ptr(arr(s.atype, np.uint8))
        q.cell = dptr(arr(s.cell, np.float64))
        q.temperature = float(s.temperature if temperature is None else temperature)
        q.seed = int(s.seed if seed is None else seed) & (2**64 - 1)
        t1, t2, td = (arr(x, dt) for x, dt in zip(s.tethers, (np.int32, np.int32, np.float64)))
        q.n_tethers, q.teth_i1, q.teth_i2, q.teth_d = len(t1), _ip(t1), _ip(t2), _dp(td)
        a1, a2, a3, at = (arr(x, dt) for x, dt in zip(s.angles, (np.int32,) * 3 + (np.float64,)))
        q.n_angles, q.ang_i1, q.ang_i2, q.ang_i3, q.ang_theta = len(a1), _ip(a1), _ip(a2), _ip(a3), _dp(at)
        d1, d2, d3, d4, dp = (arr(x, dt) for x, dt in zip(s.dihedrals, (np.int32,) * 4 + (np.float64,)))
        q.n_dihedrals = len(d1)
        q.dih_i1, q.dih_i2, q.dih_i3, q.dih_i4, q.dih_phi = _ip(d1), _ip(d2), _ip(d3), _ip(d4), _dp(dp)
        n1, n2, nd = (arr(x, dt) for x, dt in zip(s.natives, (np.int32, np.int32, np.float64)))
        q.n_natives, q.nat_i1, q.nat_i2, q.nat_d = len(n1), _ip(n1), _ip(n2), _dp(nd)
        q.r = dptr(arr(np.asarray(s.r).reshape(-1), np.float64))
        q.v = None
        q.nsteps = int(nsteps)
        rid = C.c_int64()
        check(self.lib.xmd_gpu_server_submit(self.h, C.byref(q), C.byref(rid)))
        self.sizes[rid.value] = s.n
        return rid.value

    def poll(self, rid: int) -> int:
        st = C.c_int32()
        check(self.lib.xmd_gpu_server_poll(self.h, int(rid), C.byref(st)))
        return st.value

    def result(self, rid: int):
        """Wait for a request: final positions, velocities [n, 3], time, latency (s)."""
        n = self.sizes.pop(rid)
        r, v = np.zeros(3 * n), np.zeros(3 * n)
        t, lat = C.c_double(), C.c_double()
        check(self.lib.xmd_gpu_server_result(self.h, int(rid), dptr(r), dptr(v), C.byref(t), C.byref(lat)))
        return r.reshape(n, 3), v.reshape(n, 3), t.value, lat.value

    def wait_all(self):
        check(self.lib.xmd_gpu_server_wait_all(self.h))

    def stats(self) -> dict:
        out = np.zeros(len(abi.SRV_KEYS))
        check(self.lib.xmd_gpu_server_stats(self.h, dptr(out)))
        return dict(zip(abi.SRV_KEYS, out.tolist()))
