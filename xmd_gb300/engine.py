"""Host-side handle on an engine context (thin wrapper over the C ABI).

Mirrors the way the reference drives its hot path (src/freeform/main.cpp):
parameters come from YAML, each system's topology and native structure are
handed over once, and the step loop runs on the device.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import check, dptr, iptr, u8ptr


class Engine:
    def __init__(self, yaml_text: str = ""):
        self.lib = abi.load()
        h = C.c_void_p()
        check(self.lib.xmd_gpu_create(yaml_text.encode(), C.byref(h)))
        self.h = h
        self.sizes: dict[int, int] = {}

    def close(self):
        if self.h:
            self.lib.xmd_gpu_destroy(self.h)
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

    @property
    def params(self) -> abi.Params:
        p = abi.Params()
        check(self.lib.xmd_gpu_get_params(self.h, C.byref(p)))
        return p

    def enable_term(self, term: int, on: bool = True):
        check(self.lib.xmd_gpu_enable_term(self.h, term, int(on)))

    def add_system(self, s, temperature: float | None = None, seed: int | None = None) -> int:
        """Add a synth.System (or anything with the same fields) as a replica."""
        chain = np.ascontiguousarray(s.chain, dtype=np.int32)
        seq = np.ascontiguousarray(s.seq, dtype=np.int32)
        at = np.ascontiguousarray(s.atype, dtype=np.uint8)
        cell = np.ascontiguousarray(s.cell, dtype=np.float64)
        rid = C.c_int32()
        T = s.temperature if temperature is None else temperature
        sd = s.seed if seed is None else seed
        check(self.lib.xmd_gpu_add_replica(self.h, s.n, iptr(chain), iptr(seq), u8ptr(at), dptr(cell),
                                           float(T), int(sd) & (2**64 - 1), C.byref(rid)))
        r = rid.value
        t1, t2, td = (np.ascontiguousarray(x) for x in s.tethers)
        check(self.lib.xmd_gpu_set_tethers(self.h, r, len(t1), iptr(t1), iptr(t2), dptr(td)))
        a1, a2, a3, at0 = (np.ascontiguousarray(x) for x in s.angles)
        check(self.lib.xmd_gpu_set_angles(self.h, r, len(a1), iptr(a1), iptr(a2), iptr(a3), dptr(at0)))
        d1, d2, d3, d4, dp = (np.ascontiguousarray(x) for x in s.dihedrals)
        check(self.lib.xmd_gpu_set_dihedrals(self.h, r, len(d1), iptr(d1), iptr(d2), iptr(d3), iptr(d4),
                                             dptr(dp)))
        n1, n2, nd = (np.ascontiguousarray(x) for x in s.natives)
        check(self.lib.xmd_gpu_set_native_contacts(self.h, r, len(n1), iptr(n1), iptr(n2), dptr(nd)))
        if getattr(s, "chirals", None) is not None:
            q = [np.ascontiguousarray(x, dtype=np.int32) for x in s.chirals[:4]]
            qf, qc = (np.ascontiguousarray(x, dtype=np.float64) for x in s.chirals[4:])
            check(self.lib.xmd_gpu_set_chirals(self.h, r, len(q[0]), *(iptr(x) for x in q), dptr(qf), dptr(qc)))
        if getattr(s, "ssbonds", None) is not None:
            s1, s2 = (np.ascontiguousarray(x, dtype=np.int32) for x in s.ssbonds)
            check(self.lib.xmd_gpu_set_ssbonds(self.h, r, len(s1), iptr(s1), iptr(s2)))
        if getattr(s, "afm_vel", None) is not None:
            b = np.ascontiguousarray(s.afm_vel[0], dtype=np.int32)
            o, v = (np.ascontiguousarray(x, dtype=np.float64).reshape(-1) for x in s.afm_vel[1:])
            check(self.lib.xmd_gpu_set_velocity_afm(self.h, r, len(b), iptr(b), dptr(o), dptr(v)))
        if getattr(s, "afm_force", None) is not None:
            b = np.ascontiguousarray(s.afm_force[0], dtype=np.int32)
            f = np.ascontiguousarray(s.afm_force[1], dtype=np.float64).reshape(-1)
            check(self.lib.xmd_gpu_set_force_afm(self.h, r, len(b), iptr(b), dptr(f)))
        if getattr(s, "heur_angles", None) is not None:
            h = [np.ascontiguousarray(x, dtype=np.int32) for x in s.heur_angles]
            check(self.lib.xmd_gpu_set_heuristic_angles(self.h, r, len(h[0]), *(iptr(x) for x in h)))
        if getattr(s, "heur_dihedrals", None) is not None:
            h = [np.ascontiguousarray(x, dtype=np.int32) for x in s.heur_dihedrals]
            check(self.lib.xmd_gpu_set_heuristic_dihedrals(self.h, r, len(h[0]), *(iptr(x) for x in h)))
        rr = np.ascontiguousarray(s.r, dtype=np.float64).reshape(-1)
        check(self.lib.xmd_gpu_set_state(self.h, r, dptr(rr), None))
        self.sizes[r] = s.n
        return r

    def set_walls(self, kind: int, origin, normal):
        """Wall planes of one kind (0 solid, 1 LJ attractive), before the
        first step or evaluation."""
        o = np.ascontiguousarray(origin, dtype=np.float64).reshape(-1)
        n = np.ascontiguousarray(normal, dtype=np.float64).reshape(-1)
        check(self.lib.xmd_gpu_set_walls(self.h, int(kind), len(o) // 3, dptr(o), dptr(n)))

    def eval_forces(self, rep: int = 0):
        n = self.sizes[rep]
        F = np.zeros(3 * n)
        V = np.zeros(abi.NUM_TERMS)
        check(self.lib.xmd_gpu_eval_forces(self.h, rep, dptr(F), dptr(V)))
        return F.reshape(n, 3), V

    def step(self, nsteps: int):
        check(self.lib.xmd_gpu_step(self.h, int(nsteps)))

    def get_state(self, rep: int = 0):
        n = self.sizes[rep]
        r, v, t = np.zeros(3 * n), np.zeros(3 * n), C.c_double()
        check(self.lib.xmd_gpu_get_state(self.h, rep, dptr(r), dptr(v), C.byref(t)))
        return r.reshape(n, 3), v.reshape(n, 3), t.value

    def autotune(self, steps: int = 96) -> dict:
        """Times every launch shape on a clone of this context and keeps the
        fastest (results never depend on the shape)."""
        shape = np.zeros(4, dtype=np.int32)
        ms = C.c_double()
        check(self.lib.xmd_gpu_autotune(self.h, int(steps), iptr(shape), C.byref(ms)))
        return {"fb": int(shape[0]), "tile_per_sm": int(shape[1]), "graph_steps": int(shape[2]),
                "lpb": int(shape[3]), "ms_per_step": ms.value}

    def tuning(self) -> dict:
        shape = np.zeros(4, dtype=np.int32)
        check(self.lib.xmd_gpu_get_tuning(self.h, iptr(shape)))
        return {"fb": int(shape[0]), "tile_per_sm": int(shape[1]), "graph_steps": int(shape[2]),
                "lpb": int(shape[3])}

    def set_tuning(self, fb: int, tile_per_sm: int, graph_steps: int, lpb: int = 4):
        shape = np.array([fb, tile_per_sm, graph_steps, lpb], dtype=np.int32)
        check(self.lib.xmd_gpu_set_tuning(self.h, iptr(shape)))

    def set_state(self, rep: int, r: np.ndarray, v: np.ndarray | None = None):
        r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1)
        vp = None
        if v is not None:
            v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
            vp = dptr(v)
        check(self.lib.xmd_gpu_set_state(self.h, rep, dptr(r), vp))

    def get_history(self, rep: int = 0):
        n = self.sizes[rep]
        y, t, st = np.zeros(18 * n), C.c_double(), C.c_uint64()
        check(self.lib.xmd_gpu_get_history(self.h, rep, dptr(y), C.byref(t), C.byref(st)))
        return y.reshape(6, n, 3), t.value, st.value

    def set_history(self, rep: int, y: np.ndarray, t: float, rng_state: int):
        y = np.ascontiguousarray(y, dtype=np.float64).reshape(-1)
        check(self.lib.xmd_gpu_set_history(self.h, rep, dptr(y), float(t), int(rng_state)))

    def snapshot(self, rep: int = 0) -> bytes:
        """The replica's whole mutable state (xmd_gpu_snapshot)."""
        nb = C.c_int64()
        check(self.lib.xmd_gpu_snapshot_size(self.h, rep, C.byref(nb)))
        buf = C.create_string_buffer(nb.value)
        check(self.lib.xmd_gpu_snapshot(self.h, rep, buf, nb.value))
        return buf.raw

    def restore(self, rep: int, snap: bytes):
        """Continue from a snapshot of the same replica slot (xmd_gpu_restore)."""
        buf = C.create_string_buffer(bytes(snap), len(snap))
        check(self.lib.xmd_gpu_restore(self.h, rep, buf, len(snap)))

    def observables(self, rep: int = 0):
        E, K, Rg, Q = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        check(self.lib.xmd_gpu_observables(self.h, rep, C.byref(E), C.byref(K), C.byref(Rg), C.byref(Q)))
        return {"E": E.value, "K": K.value, "Rg": Rg.value, "Q": Q.value}

    def qa_contacts(self, rep: int = 0, cap: int = 1 << 20):
        out = np.zeros(4 * cap, dtype=np.int32)
        rt = np.zeros(cap)
        m = C.c_int32()
        check(self.lib.xmd_gpu_qa_contacts(self.h, rep, cap, iptr(out), dptr(rt), C.byref(m)))
        k = min(m.value, cap)
        return out[:4 * k].reshape(k, 4), rt[:k]

    def qa_sync(self, rep: int = 0):
        out = np.zeros(4 * self.sizes[rep], dtype=np.int8)
        check(self.lib.xmd_gpu_qa_sync(self.h, rep, out.ctypes.data_as(C.POINTER(C.c_int8))))
        return out.reshape(-1, 4)

    def stats(self) -> dict:
        out = np.zeros(8, dtype=np.int64)
        check(self.lib.xmd_gpu_stats(self.h, out.ctypes.data_as(C.POINTER(C.c_int64))))
        keys = ["beads", "replicas", "nl_entries", "go_active", "rebuilds", "launches", "qa_contacts", "md_steps"]
        return dict(zip(keys, out.tolist()))

    def device_status(self) -> int:
        s = C.c_int32()
        check(self.lib.xmd_gpu_device_status(self.h, C.byref(s)))
        return s.value

    def reserve(self, beads: int, replicas: int, native_entries: int):
        """Fixed device capacities; replicas can then come and go between steps."""
        check(self.lib.xmd_gpu_reserve(self.h, int(beads), int(replicas), int(native_entries)))

    def remove_replica(self, rep: int):
        check(self.lib.xmd_gpu_remove_replica(self.h, int(rep)))
        self.sizes.pop(rep, None)

    def set_steps(self, rep: int, nsteps: int):
        check(self.lib.xmd_gpu_set_steps(self.h, int(rep), int(nsteps)))

    def steps_left(self) -> np.ndarray:
        """Per replica slot: steps still to take (-1: unbounded), -2 for a free
        slot, -3 for a replica frozen by a non-finite force."""
        n = max(self.sizes) + 1 if self.sizes else 0
        # the library writes one entry per replica slot it has handed out
        out = np.zeros(n + (1 << 16), dtype=np.int64)
        check(self.lib.xmd_gpu_steps_left(self.h, out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out[:n]

    def synchronize(self):
        check(self.lib.xmd_gpu_synchronize(self.h))
