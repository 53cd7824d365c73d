"""The allocation-free pair search against the engine's own Verlet list.

xmd_gpu_verlet_pairs_noalloc() serves callers that cannot allocate device
memory where they need a pair list (inside a CUDA graph capture, under a
fixed memory pool, in loops that cannot take cudaMalloc's synchronisation).
It reads caller-owned device buffers and keeps its scratch in a file-scope
device array shared by every call.  This test feeds it device buffers the
test allocates, calls it twice in a row on different systems (so stale
scratch from the first call would show in the second), and compares each
result with the pair list of the regular, allocating path
(xmd_gpu_verlet_pairs on an engine context holding the same system).

The systems make the two lists coincide: every bead is charged and there are
no native contacts, so the engine keeps every non-excluded pair within its
Verlet radius (the ES list's 2D + pad equals that radius), which is the set
the allocation-free search returns for cutoff = the Verlet radius.
"""
import ctypes

import numpy as np
import pytest

from tests.util import cudart
from xmd_gb300 import Engine, abi, synth

pytestmark = pytest.mark.gpu

ANGSTROM = 0.2
LYS = abi.AA.index("LYS")


def all_charged_system(chains, length, seed, box_a):
    box = None if box_a is None else box_a * ANGSTROM
    s = synth.make_system([length] * chains, seed, box=box, temperature=0.35, native=False)
    s.atype = np.full(s.n, LYS, dtype=np.uint8)
    return s


def engine_pairs(s):
    y = synth.yaml_for("c2")
    with Engine(y) as e:
        e.add_system(s)
        cap = 64 * s.n + 64
        out = np.zeros(2 * cap, dtype=np.int32)
        flags = np.zeros(cap, dtype=np.uint8)
        cnt = ctypes.c_int32()
        abi.check(e.lib.xmd_gpu_verlet_pairs(e.h, 0, cap, abi.iptr(out),
                                              flags.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                              ctypes.byref(cnt)))
    k = cnt.value
    assert (flags[:k] & 2).all()          # every kept pair is on the ES list
    return out[:2 * k].reshape(k, 2)


class DeviceBuffers:
    """Device memory owned by the caller (the test), not by the entry point."""

    def __init__(self, rt):
        self.rt = rt
        self.ptrs = []

    def put(self, arr):
        arr = np.ascontiguousarray(arr)
        p = ctypes.c_void_p()
        assert self.rt.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(max(arr.nbytes, 16))) == 0
        assert self.rt.cudaMemcpy(p, arr.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(arr.nbytes), 1) == 0
        self.ptrs.append(p)
        return p

    def empty(self, nbytes):
        p = ctypes.c_void_p()
        assert self.rt.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(max(nbytes, 16))) == 0
        self.ptrs.append(p)
        return p

    def get(self, p, dtype, count):
        out = np.zeros(count, dtype=dtype)
        assert self.rt.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), p, ctypes.c_size_t(out.nbytes), 2) == 0
        return out

    def free(self):
        for p in self.ptrs:
            self.rt.cudaFree(p)
        self.ptrs = []


def noalloc_pairs(lib, rt, bufs, s, cutoff, cap=None, want_count=False):
    d_r = bufs.put(np.asarray(s.r, dtype=np.float64).reshape(-1))
    d_chain = bufs.put(np.asarray(s.chain, dtype=np.int32))
    d_seq = bufs.put(np.asarray(s.seq, dtype=np.int32))
    cap = 64 * s.n + 64 if cap is None else cap
    d_pairs = bufs.empty(8 * cap)
    d_count = bufs.empty(4)
    cell = np.ascontiguousarray(s.cell, dtype=np.float64)
    abi.check(lib.xmd_gpu_verlet_pairs_noalloc(d_r, d_chain, d_seq, s.n, abi.dptr(cell), cutoff,
                                               d_pairs, cap, d_count, None))
    assert rt.cudaDeviceSynchronize() == 0
    total = int(bufs.get(d_count, np.int32, 1)[0])
    k = min(total, cap)
    got = bufs.get(d_pairs, np.int32, 2 * k).reshape(k, 2)
    return (got, total) if want_count else got


def test_noalloc_pairs_match_engine_two_calls():
    lib = abi.load()
    rt = cudart()
    first = all_charged_system(6, 40, 77, 70.0)       # periodic, 240 beads
    second = all_charged_system(3, 55, 78, 45.0)      # periodic, 165 beads, denser
    want1, want2 = engine_pairs(first), engine_pairs(second)
    assert len(want1) > 100 and len(want2) > 100
    verlet_radius = (20.0 + 5.0) * ANGSTROM           # 2 D + pad_factor * 2 D
    bufs = DeviceBuffers(rt)
    try:
        got1 = noalloc_pairs(lib, rt, bufs, first, verlet_radius)
        got2 = noalloc_pairs(lib, rt, bufs, second, verlet_radius)
    finally:
        bufs.free()
    # same pairs, and the allocation-free result is already in (i, j) order
    assert np.array_equal(got1, want1)
    assert np.array_equal(got2, want2)


def test_noalloc_rejects_oversize():
    lib = abi.load()
    cell = np.zeros(3)
    rc = lib.xmd_gpu_verlet_pairs_noalloc(None, None, None, abi.NOALLOC_MAX_BEADS + 1, abi.dptr(cell), 1.0,
                                          None, 0, None, None)
    assert rc == -5
    assert b"XMD_NOALLOC_MAX_BEADS" in lib.xmd_gpu_last_error()


def free_device_bytes(rt):
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def test_noalloc_open_boundary_truncation_and_no_allocation():
    """An open (non-periodic) system, where cells clamp at the low corner and
    out-of-range neighbour cells are skipped, against the engine's list; a
    call whose cap is below the pair count returns the full count and the
    first cap pairs of the (i, j)-ordered list; and repeated calls leave the
    device's free memory unchanged (no allocation behind the caller's back)."""
    lib = abi.load()
    rt = cudart()
    s = all_charged_system(4, 50, 91, None)
    assert not np.asarray(s.cell).any()
    want = engine_pairs(s)
    assert len(want) > 100
    verlet_radius = (20.0 + 5.0) * ANGSTROM
    bufs = DeviceBuffers(rt)
    try:
        got, total = noalloc_pairs(lib, rt, bufs, s, verlet_radius, want_count=True)
        assert total == len(want) and np.array_equal(got, want)
        for cap in (len(want) // 3, len(want) - 1, 1):
            part, total = noalloc_pairs(lib, rt, bufs, s, verlet_radius, cap=cap, want_count=True)
            assert total == len(want)
            assert np.array_equal(part, want[:cap])
        # buffers of the next call first, then the free memory around it
        d_r = bufs.put(np.asarray(s.r, dtype=np.float64).reshape(-1))
        d_chain = bufs.put(np.asarray(s.chain, dtype=np.int32))
        d_seq = bufs.put(np.asarray(s.seq, dtype=np.int32))
        cap = 64 * s.n
        d_pairs = bufs.empty(8 * cap)
        d_count = bufs.empty(4)
        cell = np.zeros(3)
        assert rt.cudaDeviceSynchronize() == 0
        before = free_device_bytes(rt)
        for _ in range(3):
            abi.check(lib.xmd_gpu_verlet_pairs_noalloc(d_r, d_chain, d_seq, s.n, abi.dptr(cell), verlet_radius,
                                                       d_pairs, cap, d_count, None))
        assert rt.cudaDeviceSynchronize() == 0
        assert free_device_bytes(rt) == before
        assert int(bufs.get(d_count, np.int32, 1)[0]) == len(want)
    finally:
        bufs.free()
