"""ctypes view of the C ABI in include/xmd_gpu.h.

The engine is the shared library built in-tree by xmd_gb300.build; loading
fails loudly when it is missing (there is no fallback implementation).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

NUM_TERMS = 18
NUM_AA = 20
NUM_SS = NUM_AA * NUM_AA
TERM_NAMES = ["tether", "nat_ang", "cnd", "snd", "go", "pauli", "const_es", "rel_es", "qa",
              "chir", "nat_ss", "heur_ang", "heur_dih", "vel_afm", "force_afm", "solid_wall", "lj_wall",
              "pid"]
(TERM_TETHER, TERM_NAT_ANG, TERM_CND, TERM_SND, TERM_GO, TERM_PAULI, TERM_CONST_ES,
 TERM_REL_ES, TERM_QA, TERM_CHIR, TERM_NAT_SS, TERM_HEUR_ANG, TERM_HEUR_DIH,
 TERM_VEL_AFM, TERM_FORCE_AFM, TERM_SOLID_WALL, TERM_LJ_WALL, TERM_PID) = range(NUM_TERMS)
PREC_FP64, PREC_MIXED = 0, 1
NOALLOC_MAX_BEADS = 65536   # XMD_NOALLOC_MAX_BEADS

ERRORS = {-1: "XMD_ERR_ARG", -2: "XMD_ERR_CONFIG", -3: "XMD_ERR_STATE", -4: "XMD_ERR_CUDA",
          -5: "XMD_ERR_CAPACITY", -6: "XMD_ERR_NUMERIC", -7: "XMD_ERR_BUDGET"}

# amino-acid codes of include/xmd/types/amino_acid.h:10-13
AA = ["ALA", "ARG", "ASN", "ASP", "CYS", "GLU", "GLN", "GLY", "HIS", "ILE",
      "LEU", "LYS", "MET", "PHE", "PRO", "SER", "THR", "TRP", "TYR", "VAL"]

_d = C.c_double
_i = C.c_int32


class Params(C.Structure):
    """xmd_params (include/xmd_gpu.h)."""
    _fields_ = [
        ("on", _i * NUM_TERMS), ("langevin_on", _i), ("precision", _i),
        ("total_time", _d), ("seed", C.c_uint64),
        ("gamma_factor", _d), ("temperature", _d), ("dt", _d),
        ("pad_factor", _d), ("nl_cutoff", _d), ("nl_skin", _d),
        ("tether_H1", _d), ("tether_H2", _d), ("tether_def_length", _d),
        ("nat_ang_k", _d), ("cnd_CDA", _d), ("cnd_CDB", _d), ("snd_CDH", _d),
        ("go_depth", _d), ("go_active_threshold", _d),
        ("pauli_r_excl", _d), ("pauli_depth", _d),
        ("const_es_screen_dist", _d), ("const_es_permittivity", _d),
        ("rel_es_screen_dist", _d), ("rel_es_factor", _d),
        ("charge", _d * NUM_AA), ("polarization", _i * NUM_AA), ("limits", (_i * 4) * NUM_AA),
        ("qa_phase_duration", _d), ("qa_breaking_factor", _d),
        ("qa_min_cos_hr", _d), ("qa_min_cos_hh", _d), ("qa_max_cos_nr", _d),
        ("lj_bb_r_min", _d), ("lj_bb_depth", _d), ("lj_bs_r_min", _d), ("lj_bs_depth", _d),
        ("ss_sinking", _i), ("ss_depth", _d * NUM_SS), ("ss_r_max", _d * NUM_SS),
        ("nl_capacity", _i), ("nl_grow", _i), ("device", _i), ("nl_build", _i),
        ("chir_e_chi", _d), ("nat_ss_H1", _d), ("nat_ss_dist", _d),
        ("heur_ang_coeffs", (_d * 7) * 9), ("heur_dih_coeffs", (_d * 6) * 9),
        ("vel_afm_H1", _d), ("vel_afm_H2", _d),
        ("solid_wall_depth", _d), ("solid_wall_cutoff", _d),
        ("lj_wall_min_dist", _d), ("lj_wall_breaking_factor", _d), ("lj_wall_phase_duration", _d),
        ("lj_wall_depth", _d),
        ("pid_lambda", _i), ("pid_bbp", _d * 4), ("pid_bbm", _d * 4), ("pid_ss", _d * 2),
    ]

    def copy(self) -> "Params":
        out = Params()
        C.memmove(C.byref(out), C.byref(self), C.sizeof(Params))
        return out


class Request(C.Structure):
    """xmd_request (include/xmd_gpu.h)."""
    _pi, _pdd, _pu = C.POINTER(C.c_int32), C.POINTER(C.c_double), C.POINTER(C.c_uint8)
    _fields_ = [
        ("n", _i), ("chain_idx", _pi), ("seq_idx", _pi), ("atype", _pu), ("cell", _pdd),
        ("temperature", _d), ("seed", C.c_uint64),
        ("n_tethers", _i), ("teth_i1", _pi), ("teth_i2", _pi), ("teth_d", _pdd),
        ("n_angles", _i), ("ang_i1", _pi), ("ang_i2", _pi), ("ang_i3", _pi), ("ang_theta", _pdd),
        ("n_dihedrals", _i), ("dih_i1", _pi), ("dih_i2", _pi), ("dih_i3", _pi), ("dih_i4", _pi),
        ("dih_phi", _pdd),
        ("n_natives", _i), ("nat_i1", _pi), ("nat_i2", _pi), ("nat_d", _pdd),
        ("r", _pdd), ("v", _pdd), ("nsteps", C.c_int64),
    ]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, -1
SRV_KEYS = ["p50_s", "p99_s", "bead_steps_per_s", "completed", "queued", "running", "chunks", "peak_running",
            "cap_beads", "bead_steps", "span_s", "failed", "device_bytes", "budget_bytes", "bytes_per_bead",
            "admit_s", "step_s"]

LIB_PATH = Path(__file__).resolve().parent / "libxmdgpu.so"

P = C.POINTER
_pd, _pi32, _pu8, _pu64 = P(C.c_double), P(C.c_int32), P(C.c_uint8), P(C.c_uint64)

# (name, restype, argtypes) for every entry point of include/xmd_gpu.h
SIGNATURES = [
    ("xmd_gpu_abi_version", C.c_int, []),
    ("xmd_gpu_params_size", C.c_int, []),
    ("xmd_gpu_last_error", C.c_char_p, []),
    ("xmd_gpu_rng_jump", C.c_uint64, [C.c_uint64, C.c_uint64]),
    ("xmd_gpu_parse_params", C.c_int, [C.c_char_p, P(Params)]),
    ("xmd_gpu_create", C.c_int, [C.c_char_p, P(C.c_void_p)]),
    ("xmd_gpu_create_from_file", C.c_int, [C.c_char_p, P(C.c_void_p)]),
    ("xmd_gpu_destroy", C.c_int, [C.c_void_p]),
    ("xmd_gpu_get_params", C.c_int, [C.c_void_p, P(Params)]),
    ("xmd_gpu_set_params", C.c_int, [C.c_void_p, P(Params)]),
    ("xmd_gpu_enable_term", C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    ("xmd_gpu_set_precision", C.c_int, [C.c_void_p, C.c_int]),
    ("xmd_gpu_add_replica", C.c_int, [C.c_void_p, C.c_int32, _pi32, _pi32, _pu8, _pd, C.c_double,
                                      C.c_uint64, _pi32]),
    ("xmd_gpu_set_tethers", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _pi32, _pi32, _pd]),
    ("xmd_gpu_set_angles", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _pi32, _pi32, _pi32, _pd]),
    ("xmd_gpu_set_dihedrals", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _pi32, _pi32, _pi32, _pi32,
                                        _pd]),
    ("xmd_gpu_set_native_contacts", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _pi32, _pi32, _pd]),
    ("xmd_gpu_set_chirals", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _pi32, _pi32, _pi32, _pi32, _pd, _pd]),
    ("xmd_gpu_set_ssbonds", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _pi32, _pi32]),
    ("xmd_gpu_set_velocity_afm", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _pi32, _pd, _pd]),
    ("xmd_gpu_set_force_afm", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _pi32, _pd]),
    ("xmd_gpu_set_walls", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _pd, _pd]),
    ("xmd_gpu_set_heuristic_angles", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _pi32, _pi32, _pi32]),
    ("xmd_gpu_set_heuristic_dihedrals", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _pi32, _pi32, _pi32, _pi32]),
    ("xmd_gpu_set_state", C.c_int, [C.c_void_p, C.c_int32, _pd, _pd]),
    ("xmd_gpu_set_history", C.c_int, [C.c_void_p, C.c_int32, _pd, C.c_double, C.c_uint64]),
    ("xmd_gpu_get_state", C.c_int, [C.c_void_p, C.c_int32, _pd, _pd, _pd]),
    ("xmd_gpu_get_history", C.c_int, [C.c_void_p, C.c_int32, _pd, _pd, _pu64]),
    ("xmd_gpu_snapshot_size", C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int64)]),
    ("xmd_gpu_snapshot", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64]),
    ("xmd_gpu_restore", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64]),
    ("xmd_gpu_eval_forces", C.c_int, [C.c_void_p, C.c_int32, _pd, _pd]),
    ("xmd_gpu_step", C.c_int, [C.c_void_p, C.c_int32]),
    ("xmd_gpu_observables", C.c_int, [C.c_void_p, C.c_int32, _pd, _pd, _pd, _pd]),
    ("xmd_gpu_device_status", C.c_int, [C.c_void_p, _pi32]),
    ("xmd_gpu_qa_contacts", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _pi32, _pd, _pi32]),
    ("xmd_gpu_qa_sync", C.c_int, [C.c_void_p, C.c_int32, P(C.c_int8)]),
    ("xmd_gpu_verlet_pairs", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _pi32, _pu8, _pi32]),
    ("xmd_gpu_verlet_pairs_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, _pd, C.c_double,
                                               C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    ("xmd_gpu_upload_history_all", C.c_int, [C.c_void_p, _pd]),
    ("xmd_gpu_download_positions_all", C.c_int, [C.c_void_p, _pd]),
    ("xmd_gpu_download_history_all", C.c_int, [C.c_void_p, _pd]),
    ("xmd_gpu_get_stream", C.c_int, [C.c_void_p, P(C.c_void_p)]),
    ("xmd_gpu_stats", C.c_int, [C.c_void_p, P(C.c_int64)]),
    ("xmd_gpu_set_kernel_timing", C.c_int, [C.c_void_p, C.c_int]),
    ("xmd_gpu_autotune", C.c_int, [C.c_void_p, C.c_int32, _pi32, _pd]),
    ("xmd_gpu_set_tuning", C.c_int, [C.c_void_p, _pi32]),
    ("xmd_gpu_get_tuning", C.c_int, [C.c_void_p, _pi32]),
    ("xmd_gpu_kernel_times", C.c_int, [C.c_void_p, _pd, P(C.c_int64), _pd, P(C.c_int64)]),
    ("xmd_gpu_synchronize", C.c_int, [C.c_void_p]),
    ("xmd_gpu_reserve", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    ("xmd_gpu_remove_replica", C.c_int, [C.c_void_p, C.c_int32]),
    ("xmd_gpu_set_steps", C.c_int, [C.c_void_p, C.c_int32, C.c_int64]),
    ("xmd_gpu_steps_left", C.c_int, [C.c_void_p, P(C.c_int64)]),
    ("xmd_gpu_server_create", C.c_int, [C.c_char_p, C.c_int64, C.c_int32, C.c_int32, P(C.c_void_p)]),
    ("xmd_gpu_server_submit", C.c_int, [C.c_void_p, P(Request), P(C.c_int64)]),
    ("xmd_gpu_server_poll", C.c_int, [C.c_void_p, C.c_int64, _pi32]),
    ("xmd_gpu_server_result", C.c_int, [C.c_void_p, C.c_int64, _pd, _pd, _pd, _pd]),
    ("xmd_gpu_server_wait_all", C.c_int, [C.c_void_p]),
    ("xmd_gpu_server_stats", C.c_int, [C.c_void_p, _pd]),
    ("xmd_gpu_server_destroy", C.c_int, [C.c_void_p]),
]

_lib = None


def load(path: Path | None = None):
    """Load the engine library (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: build it with `python -m xmd_gb300.build`")
    lib = C.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.xmd_gpu_params_size() != C.sizeof(Params):
        raise RuntimeError("xmd_params layout mismatch between library and bindings")
    if path is None:
        _lib = lib
    return lib


class XmdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def check(rc: int) -> None:
    if rc != 0:
        raise XmdError(rc, load().xmd_gpu_last_error().decode())


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_pd)


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_pi32)


def u8ptr(a: np.ndarray):
    return a.ctypes.data_as(_pu8)


def parse_params(yaml_text: str = "") -> Params:
    """Resolved parameters of YAML overrides merged over the defaults (no GPU)."""
    p = Params()
    check(load().xmd_gpu_parse_params(yaml_text.encode(), C.byref(p)))
    return p
