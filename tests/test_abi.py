"""The C ABI without a GPU: every entry point that include/xmd_gpu.h declares
is exported by the library and bound by the ctypes layer with the same arity;
the parameter layout matches; the configuration layer resolves the
reference's YAML keys and units; the generator jump-ahead agrees with a direct
restatement of rand_gen (rand_gen.h:22-28)."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from xmd_gb300 import abi

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "xmd_gpu.h"


def declared():
    """(name, number of parameters) of every function the header declares."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(xmd_gpu_\w+)\s*\(([^)]*)\)\s*;", text):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_header_declares_the_boundary():
    d = declared()
    for name in ("xmd_gpu_create", "xmd_gpu_eval_forces", "xmd_gpu_step", "xmd_gpu_get_state",
                 "xmd_gpu_observables", "xmd_gpu_verlet_pairs_noalloc"):
        assert name in d


def test_library_exports_every_declared_symbol():
    lib = abi.load()
    nm = subprocess.run(["nm", "-D", "--defined-only", str(abi.LIB_PATH)], capture_output=True, text=True)
    exported = set(re.findall(r"\s(xmd_gpu_\w+)$", nm.stdout, flags=re.M)) if nm.returncode == 0 else None
    bound = {name: len(args) for name, _, args in abi.SIGNATURES}
    for name, nargs in declared().items():
        assert hasattr(lib, name), name
        if exported is not None:
            assert name in exported, name
        assert name in bound, f"{name} has no ctypes signature"
        assert bound[name] == nargs, (name, bound[name], nargs)


def test_params_layout_and_version():
    lib = abi.load()
    assert lib.xmd_gpu_params_size() == C.sizeof(abi.Params)
    assert lib.xmd_gpu_abi_version() >= 1


def test_defaults_and_units():
    p = abi.parse_params("")
    # defaults.yml: tether H1 100 eps/A^2, r_excl 4 A, const ES 10 A / 80 eps_0 (internal units, A = 0.2)
    assert p.tether_H1 == pytest.approx(100.0 / 0.04)
    assert p.pauli_r_excl == pytest.approx(0.8)
    assert p.const_es_screen_dist == pytest.approx(2.0)
    assert p.dt == pytest.approx(0.005)
    assert p.precision == abi.PREC_FP64 and p.nl_build == 0 and p.nl_grow == 1
    q = abi.parse_params("Pauli exclusion:\n  r_excl: 5.0 A\nengine:\n  precision: mixed\n  nl build: tile\n"
                         "neighbor list:\n  cutoff: 18 A\n  skin: 2 A\n")
    assert q.pauli_r_excl == pytest.approx(1.0)
    assert q.precision == abi.PREC_MIXED and q.nl_build == 2
    assert q.nl_cutoff == pytest.approx(3.6) and q.nl_skin == pytest.approx(0.4)
    # sections merge key by key over the defaults: other Pauli keys keep their values
    assert q.pauli_depth == p.pauli_depth


@pytest.mark.parametrize("text", ["engine:\n  precision: fp16\n", "engine:\n  nl build: grid\n",
                                  "integrator:\n  dt: banana\n"])
def test_bad_config_is_an_error_not_a_crash(text):
    with pytest.raises(abi.XmdError) as ei:
        abi.parse_params(text)
    assert ei.value.code in (-1, -2)


def _xs_step(s):
    m = (1 << 64) - 1
    s ^= s >> 11
    s ^= (s << 31) & m
    s ^= s >> 18
    return s


@pytest.mark.parametrize("draws", [0, 1, 4, 400, 4 * 77663])
def test_rng_jump_equals_repeated_draws(draws):
    lib = abi.load()
    seed = 0x9E3779B97F4A7C15
    s = seed
    for _ in range(draws):
        s = _xs_step(s)
    assert lib.xmd_gpu_rng_jump(seed, draws) == s
