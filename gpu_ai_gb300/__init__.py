"""GB300-native Monte Carlo playout engine for 8x8 checkers.

The compute path is libgpuai.so (hand-written sm_103a CUDA kernels behind the
C ABI in include/gpuai.h); :class:`Engine` is its Python binding.
"""
from .engine import (  # noqa: F401
    ERR_CUDA,
    ERR_INVALID,
    ERR_LIMIT,
    ERR_NO_DEVICE,
    ERR_OOM,
    LAYOUT_THREAD,
    LAYOUT_WARP,
    LAYOUT_POOLED,
    OK,
    POLICY_EPS_GREEDY,
    POLICY_RANDOM,
    POLICY_REF_HEURISTIC,
    START_BOARD,
    Engine,
    Net,
    Searches,
    GpuAIError,
    header_symbols,
    load_library,
)

__all__ = [
    "Engine",
    "Net",
    "Searches",
    "GpuAIError",
    "load_library",
    "header_symbols",
    "START_BOARD",
    "POLICY_RANDOM",
    "POLICY_REF_HEURISTIC",
    "POLICY_EPS_GREEDY",
    "LAYOUT_THREAD",
    "LAYOUT_WARP",
    "LAYOUT_POOLED",
]
