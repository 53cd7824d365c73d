"""GB300 engine for XMD's per-step hot path (Verlet build, pair and bonded
forces, Langevin predictor-corrector), driven through the C ABI of
include/xmd_gpu.h."""
from . import abi, synth
from .abi import parse_params, XmdError
from .engine import Engine
from .server import Server

__all__ = ["abi", "synth", "parse_params", "XmdError", "Engine", "Server"]
