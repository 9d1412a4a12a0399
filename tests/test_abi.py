"""The C-ABI library builds for sm_103a, loads, and exports what include/gpuai.h declares."""
import ctypes
import os
import subprocess

import pytest

from gpu_ai_gb300 import engine as E

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_library_exports_header(lib_built):
    lib = E.load_library()
    names = E.header_symbols()
    assert {"gpuai_create", "gpuai_playouts", "gpuai_genmoves", "gpuai_random_positions"} <= set(names)
    for n in names:
        assert hasattr(lib, n), n
    nm = subprocess.run(["nm", "-D", "--defined-only", lib_built], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in nm.splitlines() if " T " in line}
    assert set(names) <= exported


def test_struct_layout(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(
        '#include "gpuai.h"\n#include <stddef.h>\n'
        "_Static_assert(sizeof(gpuai_board) == 16, \"board\");\n"
        "_Static_assert(sizeof(gpuai_move) == 32, \"move\");\n"
        "_Static_assert(offsetof(gpuai_move, path) == 4, \"path\");\n"
        "_Static_assert(offsetof(gpuai_move, removed) == 16, \"removed\");\n"
        "int main(void) { return 0; }\n")
    subprocess.run(["gcc", "-std=c11", "-I" + os.path.join(ROOT, "include"), "-c", str(src), "-o",
                    str(tmp_path / "layout.o")], check=True)


def test_kernels_are_sm103a(lib_built):
    out = subprocess.run(["cuobjdump", "--list-elf", lib_built], capture_output=True, text=True).stdout
    assert "sm_103a" in out


def _gpu_present():
    try:
        lib = E.load_library()
        ctx = ctypes.c_void_p()
        rc = lib.gpuai_create(0, ctypes.byref(ctx))
        if rc == 0:
            lib.gpuai_destroy(ctx)
            return True
    except OSError:
        pass
    return False


def test_errors_without_device(lib_built):
    if _gpu_present():
        pytest.skip("a GPU is present")
    with pytest.raises(E.GpuAIError) as ei:
        E.Engine(0)
    assert ei.value.code == E.ERR_NO_DEVICE
    assert "device" in str(ei.value)


def test_null_context_is_rejected(lib_built):
    lib = E.load_library()
    assert lib.gpuai_playouts(None, None, None, 1, 0, 0, 0, None) == E.ERR_INVALID
    assert b"ctx" in lib.gpuai_last_error()
    assert lib.gpuai_genmoves(None, None, 1, None, 1, None) == E.ERR_INVALID


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(RuntimeError):
        _fresh_load(str(tmp_path / "nope.so"))


def _fresh_load(path):
    saved = E._lib
    E._lib = None
    try:
        return E.load_library(path)
    finally:
        E._lib = saved


def test_apply_move_equals_the_oracle(lib_built):
    """gpuai_apply_move (host, no device) against the oracle's State::move on
    every legal move of seeded positions."""
    import numpy as np

    import oracle_lib as L
    boards = L.random_positions(77, 1000, 0, 80)
    moves, counts = L.genmoves(boards)
    checked = 0
    for i in range(len(boards)):
        for m in range(int(counts[i])):
            want = boards[i:i + 1].copy()
            assert L.oracle().or_apply_packed_b16(L._ptr(want, L._u32p),
                                                  L._ptr(np.ascontiguousarray(moves[i, m]), L._u8p)) == 0
            got = E.apply_move(boards[i], moves[i, m])
            assert np.array_equal(got, want[0]), (i, m)
            checked += 1
    assert checked > 2000
    bad = np.zeros(32, np.uint8)
    bad[0] = 40  # from square out of range
    with pytest.raises(E.GpuAIError):
        E.apply_move(boards[0], bad)


def test_checked_build_exports_header():
    """The bounds-checked build (-DGPUAI_CHECKS) compiles and exports the same
    entry points."""
    from gpu_ai_gb300.build import build
    so = build(checks=True)
    names = E.header_symbols()
    nm = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in nm.splitlines() if " T " in line}
    assert set(names) <= exported
