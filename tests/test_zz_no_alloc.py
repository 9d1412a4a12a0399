"""gpuai_playouts_noalloc: playouts for callers that may not allocate device
memory (a server that has reserved all device memory for its search trees,
or a move loop with a hard deadline that must not wait on the allocator).

The entry point keeps its work counter, status word and repetition prefix
sums in one statically allocated array per GPU instead of cudaMalloc'd
buffers.  It is called here through the C ABI on caller-owned device buffers
and must give exactly what the allocating gpuai_playouts gives for the same
seeds, on two calls in a row (the second reuses the array the first left
behind).  This file is collected last so that a stop at the first failure
has already run every other test."""
import ctypes

import numpy as np
import pytest

from gpu_ai_gb300 import ERR_INVALID, OK, load_library

pytestmark = pytest.mark.gpu

_u32p = ctypes.POINTER(ctypes.c_uint32)


def _noalloc(lib):
    fn = lib.gpuai_playouts_noalloc
    fn.argtypes = [ctypes.c_void_p, _u32p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32,
                   ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


@pytest.mark.parametrize("policy", [0, 1, 2])
def test_noalloc_matches_allocating_entry_point(engine, policy):
    torch = pytest.importorskip("torch")
    lib = load_library()
    fn = _noalloc(lib)
    pos = engine.random_positions(4242, 300, 0, 40)
    reps = np.random.default_rng(policy).integers(0, 50, len(pos)).astype(np.uint32)
    reps[:2] = 0
    total = int(reps.sum())
    d_pos = torch.from_numpy(pos.view(np.int32).copy()).cuda()
    d_out = torch.empty(total, dtype=torch.int8, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        seed = 1000 + call
        expected = engine.playouts(pos, reps, seed=seed, stream_base=77, policy=policy)
        d_out.fill_(5)
        torch.cuda.synchronize()
        rc = fn(d_pos.data_ptr(), reps.ctypes.data_as(_u32p), len(pos), seed, 77, policy, d_out.data_ptr(), None)
        assert rc == OK, lib.gpuai_last_error()
        np.testing.assert_array_equal(d_out.cpu().numpy(), expected)


def test_noalloc_one_playout_per_board_and_limit(engine):
    torch = pytest.importorskip("torch")
    lib = load_library()
    fn = _noalloc(lib)
    pos = engine.random_positions(7, 500, 0, 30)
    d_pos = torch.from_numpy(pos.view(np.int32).copy()).cuda()
    d_out = torch.empty(len(pos), dtype=torch.int8, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        assert fn(d_pos.data_ptr(), None, len(pos), 3 + call, 0, 0, d_out.data_ptr(), None) == OK
        np.testing.assert_array_equal(d_out.cpu().numpy(), engine.playouts(pos, None, seed=3 + call))
    too_many = 16384 + 1
    assert fn(d_pos.data_ptr(), None, too_many, 1, 0, 0, d_out.data_ptr(), None) == ERR_INVALID
    assert b"maximum" in lib.gpuai_last_error()


def test_noalloc_at_the_maximum_position_count(engine):
    """Exactly GPUAI_NOALLOC_MAX_POSITIONS positions: the last prefix-sum word
    of the static array is used."""
    torch = pytest.importorskip("torch")
    lib = load_library()
    fn = _noalloc(lib)
    npos = 16384
    pos = engine.random_positions(99, npos, 0, 40)
    reps = np.random.default_rng(9).integers(0, 4, npos).astype(np.uint32)
    reps[-1] = 3
    total = int(reps.sum())
    d_pos = torch.from_numpy(pos.view(np.int32).copy()).cuda()
    d_out = torch.empty(total, dtype=torch.int8, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        expected = engine.playouts(pos, reps, seed=50 + call, stream_base=5, policy=call)
        rc = fn(d_pos.data_ptr(), reps.ctypes.data_as(_u32p), npos, 50 + call, 5, call, d_out.data_ptr(), None)
        assert rc == OK, lib.gpuai_last_error()
        np.testing.assert_array_equal(d_out.cpu().numpy(), expected)
