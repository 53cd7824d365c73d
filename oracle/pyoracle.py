"""Python handle on the CPU oracles (TEST INFRASTRUCTURE ONLY).

Two libraries share one flat API (oracle/xmd_oracle.h):
  * liboracle.so (prefix xo_): the C restatement in oracle/xmd_oracle.c;
  * _ref/libxmdref64.so (prefix xr_): the reference's own translation units,
    FP64 build, compiled from the reference tree by oracle/ref/build_ref.sh
    (only where that tree exists).
Only tests, the smoke check and bench.py's CPU baseline use this module.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libxmdref64.so"

_pd, _pi, _pu8, _pu64, _pi64, _pi8 = (C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_uint8),
                                      C.POINTER(C.c_uint64), C.POINTER(C.c_int64), C.POINTER(C.c_int8))
_libs: dict = {}


def _load(path: Path, pfx: str, params_type):
    key = (str(path), pfx)
    if key in _libs:
        return _libs[key]
    if not path.exists():
        raise FileNotFoundError(f"{path} is missing (build it with python -m xmd_gb300.build)")
    lib = C.CDLL(str(path))
    sig = {
        "create": (C.c_void_p, [C.POINTER(params_type), C.c_int32, _pi, _pi, _pu8, _pd, C.c_double, C.c_uint64]),
        "destroy": (None, [C.c_void_p]),
        "set_tethers": (C.c_int, [C.c_void_p, C.c_int32, _pi, _pi, _pd]),
        "set_angles": (C.c_int, [C.c_void_p, C.c_int32, _pi, _pi, _pi, _pd]),
        "set_dihedrals": (C.c_int, [C.c_void_p, C.c_int32, _pi, _pi, _pi, _pi, _pd]),
        "set_native_contacts": (C.c_int, [C.c_void_p, C.c_int32, _pi, _pi, _pd]),
        "set_chirals": (C.c_int, [C.c_void_p, C.c_int32, _pi, _pi, _pi, _pi, _pd, _pd]),
        "set_ssbonds": (C.c_int, [C.c_void_p, C.c_int32, _pi, _pi]),
        "set_heuristic_angles": (C.c_int, [C.c_void_p, C.c_int32, _pi, _pi, _pi]),
        "set_velocity_afm": (C.c_int, [C.c_void_p, C.c_int32, _pi, _pd, _pd]),
        "set_force_afm": (C.c_int, [C.c_void_p, C.c_int32, _pi, _pd]),
        "set_walls": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _pd, _pd]),
        "set_heuristic_dihedrals": (C.c_int, [C.c_void_p, C.c_int32, _pi, _pi, _pi, _pi]),
        "set_state": (C.c_int, [C.c_void_p, _pd, _pd]),
        "set_history": (C.c_int, [C.c_void_p, _pd, C.c_double, C.c_uint64]),
        "get_state": (C.c_int, [C.c_void_p, _pd, _pd, _pd]),
        "get_history": (C.c_int, [C.c_void_p, _pd, _pd, _pu64]),
        "eval_forces": (C.c_int, [C.c_void_p, _pd, _pd]),
        "step": (C.c_int, [C.c_void_p, C.c_int32]),
        "counts": (C.c_int, [C.c_void_p, _pi64]),
        "qa_contacts": (C.c_int, [C.c_void_p, C.c_int32, _pi, _pd]),
        "nl_pairs": (C.c_int, [C.c_void_p, C.c_int64, _pi]),
        "sync": (C.c_int, [C.c_void_p, _pi8]),
        "cutoffs": (C.c_int, [C.c_void_p, _pd]),
        "rng_next": (C.c_uint64, [_pu64]),
        "rng_normal": (C.c_double, [_pu64]),
    }
    if pfx == "xo_":
        sig["step_omp"] = (C.c_int, [C.c_void_p, C.c_int32, C.c_int32])
        sig["observables"] = (C.c_int, [C.c_void_p, _pd, _pd, _pd, _pd])
        sig["free_pairs"] = (C.c_int, [C.c_void_p, C.c_int32, _pi])
    for name, (res, args) in sig.items():
        fn = getattr(lib, pfx + name)
        fn.restype = res
        fn.argtypes = args
    _libs[key] = lib
    return lib


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(_pd)


class Oracle:
    """One system on a CPU oracle.  kind: 'port' (C restatement) or 'ref'
    (the reference's compiled kernels)."""

    def __init__(self, params, system, kind: str = "port", temperature=None, seed=None, walls=None):
        """walls: {kind: (origin[k, 3], normal[k, 3])}, kind 0 solid, 1 LJ attractive."""
        from xmd_gb300.abi import Params
        self.kind = kind
        self.pfx = "xo_" if kind == "port" else "xr_"
        self.lib = _load(PORT_LIB if kind == "port" else REF_LIB, self.pfx, Params)
        s = system
        self.n = s.n
        self._keep = []
        keep = lambda a, dt: self._keep.append(np.ascontiguousarray(a, dtype=dt)) or self._keep[-1]
        chain, seq, at, cell = keep(s.chain, np.int32), keep(s.seq, np.int32), keep(s.atype, np.uint8), \
            keep(s.cell, np.float64)
        T = s.temperature if temperature is None else temperature
        sd = s.seed if seed is None else seed
        self.h = self.fn("create")(C.byref(params), s.n, chain.ctypes.data_as(_pi), seq.ctypes.data_as(_pi),
                                   at.ctypes.data_as(_pu8), cell.ctypes.data_as(_pd), float(T),
                                   int(sd) & (2**64 - 1))
        if not self.h:
            raise RuntimeError("oracle create failed")
        ip = lambda a: keep(a, np.int32).ctypes.data_as(_pi)
        dp = lambda a: keep(a, np.float64).ctypes.data_as(_pd)
        t = s.tethers
        self.fn("set_tethers")(self.h, len(t[0]), ip(t[0]), ip(t[1]), dp(t[2]))
        a = s.angles
        self.fn("set_angles")(self.h, len(a[0]), ip(a[0]), ip(a[1]), ip(a[2]), dp(a[3]))
        d = s.dihedrals
        self.fn("set_dihedrals")(self.h, len(d[0]), ip(d[0]), ip(d[1]), ip(d[2]), ip(d[3]), dp(d[4]))
        nc = s.natives
        self.fn("set_native_contacts")(self.h, len(nc[0]), ip(nc[0]), ip(nc[1]), dp(nc[2]))
        q = getattr(s, "chirals", None)
        if q is not None:
            self.fn("set_chirals")(self.h, len(q[0]), ip(q[0]), ip(q[1]), ip(q[2]), ip(q[3]), dp(q[4]), dp(q[5]))
        b = getattr(s, "ssbonds", None)
        if b is not None:
            self.fn("set_ssbonds")(self.h, len(b[0]), ip(b[0]), ip(b[1]))
        a = getattr(s, "afm_vel", None)
        if a is not None:
            # a NaN origin is the bead's start position (main.cpp:884)
            o = np.array(a[1], dtype=np.float64).reshape(-1, 3)
            start = np.asarray(s.r, dtype=np.float64).reshape(-1, 3)[np.asarray(a[0])]
            o = np.where(np.isnan(o), start, o)
            self.fn("set_velocity_afm")(self.h, len(a[0]), ip(a[0]), dp(o.reshape(-1)),
                                        dp(np.asarray(a[2]).reshape(-1)))
        a = getattr(s, "afm_force", None)
        if a is not None:
            self.fn("set_force_afm")(self.h, len(a[0]), ip(a[0]), dp(np.asarray(a[1]).reshape(-1)))
        for wk, (wo, wn) in (walls or {}).items():
            if self.fn("set_walls")(self.h, int(wk), len(wo), dp(np.asarray(wo).reshape(-1)),
                                    dp(np.asarray(wn).reshape(-1))) != 0:
                raise ValueError("bad walls")
        h = getattr(s, "heur_angles", None)
        if h is not None:
            self.fn("set_heuristic_angles")(self.h, len(h[0]), ip(h[0]), ip(h[1]), ip(h[2]))
        h = getattr(s, "heur_dihedrals", None)
        if h is not None:
            self.fn("set_heuristic_dihedrals")(self.h, len(h[0]), ip(h[0]), ip(h[1]), ip(h[2]), ip(h[3]))
        self.fn("set_state")(self.h, dp(np.asarray(s.r).reshape(-1)), None)

    def fn(self, name):
        return getattr(self.lib, self.pfx + name)

    def close(self):
        if self.h:
            self.fn("destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def eval_forces(self):
        F = np.zeros(3 * self.n)
        from xmd_gb300.abi import NUM_TERMS
        V = np.zeros(NUM_TERMS)
        self.fn("eval_forces")(self.h, F.ctypes.data_as(_pd), V.ctypes.data_as(_pd))
        return F.reshape(self.n, 3), V

    def eval_at(self, r):
        """Forces and energies at positions r with the current lists (port only)."""
        from xmd_gb300.abi import NUM_TERMS
        fn = self.lib.xo_eval_at
        fn.restype, fn.argtypes = C.c_int, [C.c_void_p, _pd, _pd, _pd]
        rr = np.ascontiguousarray(r, dtype=np.float64).reshape(-1)
        F, V = np.zeros(3 * self.n), np.zeros(NUM_TERMS)
        fn(self.h, rr.ctypes.data_as(_pd), F.ctypes.data_as(_pd), V.ctypes.data_as(_pd))
        return F.reshape(self.n, 3), V

    def step(self, nsteps: int):
        self.fn("step")(self.h, int(nsteps))

    def step_omp(self, nsteps: int, nthreads: int = 0):
        self.fn("step_omp")(self.h, int(nsteps), int(nthreads))

    def get_state(self):
        r, v, t = np.zeros(3 * self.n), np.zeros(3 * self.n), C.c_double()
        self.fn("get_state")(self.h, r.ctypes.data_as(_pd), v.ctypes.data_as(_pd), C.byref(t))
        return r.reshape(self.n, 3), v.reshape(self.n, 3), t.value

    def get_history(self):
        y, t, st = np.zeros(18 * self.n), C.c_double(), C.c_uint64()
        self.fn("get_history")(self.h, y.ctypes.data_as(_pd), C.byref(t), C.byref(st))
        return y.reshape(6, self.n, 3), t.value, st.value

    def set_history(self, y, t, rng_state):
        y = np.ascontiguousarray(y, dtype=np.float64).reshape(-1)
        self.fn("set_history")(self.h, y.ctypes.data_as(_pd), float(t), int(rng_state))

    def counts(self):
        c = np.zeros(8, dtype=np.int64)
        self.fn("counts")(self.h, c.ctypes.data_as(_pi64))
        return dict(zip(["go", "pauli", "es", "free", "free_slots", "contacts", "contact_slots", "rebuilds"],
                        c.tolist()))

    def qa_contacts(self, cap=1 << 20):
        out = np.zeros(4 * cap, dtype=np.int32)
        rt = np.zeros(cap)
        m = self.fn("qa_contacts")(self.h, cap, out.ctypes.data_as(_pi), rt.ctypes.data_as(_pd))
        return out[:4 * m].reshape(m, 4), rt[:m]

    def nl_pairs(self, cap=1 << 24):
        out = np.zeros(2 * cap, dtype=np.int32)
        m = self.fn("nl_pairs")(self.h, cap, out.ctypes.data_as(_pi))
        return out[:2 * m].reshape(m, 2)

    def sync(self):
        out = np.zeros(4 * self.n, dtype=np.int8)
        self.fn("sync")(self.h, out.ctypes.data_as(_pi8))
        return out.reshape(self.n, 4)

    def cutoffs(self):
        out = np.zeros(3)
        self.fn("cutoffs")(self.h, out.ctypes.data_as(_pd))
        return out

    def observables(self):
        E, K, Rg, Q = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        self.fn("observables")(self.h, C.byref(E), C.byref(K), C.byref(Rg), C.byref(Q))
        return {"E": E.value, "K": K.value, "Rg": Rg.value, "Q": Q.value}


def parse_params(yaml_text: str = ""):
    """xmd_params of YAML overrides merged over the defaults, resolved by the
    parser linked into liboracle.so (the engine library is not loaded)."""
    from xmd_gb300.abi import Params, XmdError
    lib = _load(PORT_LIB, "xo_", Params)
    fn = lib.xo_parse_params
    fn.restype, fn.argtypes = C.c_int, [C.c_char_p, C.POINTER(Params)]
    lib.xo_last_error.restype = C.c_char_p
    p = Params()
    rc = fn(yaml_text.encode(), C.byref(p))
    if rc != 0:
        raise XmdError(rc, lib.xo_last_error().decode())
    return p


def rng_stream(kind: str, state: int, n: int):
    """n raw outputs of the reference generator from `state`."""
    from xmd_gb300.abi import Params
    lib = _load(PORT_LIB if kind == "port" else REF_LIB, "xo_" if kind == "port" else "xr_", Params)
    fn = getattr(lib, ("xo_" if kind == "port" else "xr_") + "rng_next")
    st = C.c_uint64(state)
    return np.array([fn(C.byref(st)) for _ in range(n)], dtype=np.uint64), st.value


def ref_morph_into_saw(lens, bond, density, infer_box, seed):
    """model::morph_into_saw of the reference itself (its model.cpp compiled
    into the reference driver): (r[n, 3], generator state after, cell[3])."""
    from xmd_gb300.abi import Params
    lib = _load(REF_LIB, "xr_", Params)
    fn = lib.xr_morph_into_saw
    fn.restype = C.c_int
    fn.argtypes = [C.c_int32, _pi, C.c_double, C.c_double, C.c_int32, C.c_uint64, _pd, _pu64, _pd]
    L = np.ascontiguousarray(lens, dtype=np.int32)
    n = int(L.sum())
    r = np.zeros(3 * max(n, 1))
    cell = np.zeros(3)
    st = np.zeros(1, dtype=np.uint64)
    fn(len(L), L.ctypes.data_as(_pi), float(bond if bond is not None else 0.0), float(density), int(infer_box),
       int(seed) & (2**64 - 1), r.ctypes.data_as(_pd), st.ctypes.data_as(_pu64), cell.ctypes.data_as(_pd))
    return r[:3 * n].reshape(n, 3), int(st[0]), cell
