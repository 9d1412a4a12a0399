"""The PlayoutDriver adapter a maintainer adds to the reference
(include/adapters/gpuPlayout.cpp) compiles
against the reference's own headers (src/playout.hpp:27-33,
src/state.hpp), converts the reference's starting State to the engine's
start board, and reports a missing GPU as std::runtime_error instead of
exiting.  Runs where the reference sources are present (the build machine);
skipped elsewhere."""
import os
import re
import subprocess

import pytest

import oracle_lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "gpu_ai_gb300", "lib")

MAIN = r'''
#include <cstdio>
int main() {
  const gpuai_board b = toBoard(getStartingState());
  std::printf("board %08x %08x %08x %08x\n", b.p1, b.p2, b.kings, b.meta);
  try {
    GpuPlayoutDriver d;
    std::printf("driver %s\n", d.getName().c_str());
    std::vector<State> none;
    std::printf("empty %zu\n", d.runPlayouts(none).size());
  } catch (const std::runtime_error &e) {
    std::printf("error %s\n", e.what());
  }
  return 0;
}
'''


ADAPTER = os.path.join(ROOT, "include", "adapters", "gpuPlayout.cpp")


@pytest.fixture(scope="module")
def adapter_exe(tmp_path_factory):
    if not os.path.isdir(L.REF_SRC):
        pytest.skip("reference sources not present")
    if not os.path.exists(L.REF_SO) and not L.build_ref():
        pytest.skip("reference library not built")
    if not os.path.exists(os.path.join(LIB, "libgpuai.so")):
        pytest.skip("libgpuai.so not built")
    d = tmp_path_factory.mktemp("adapter")
    (d / "main.cpp").write_text('#include "' + ADAPTER + '"\n' + MAIN)
    exe = d / "adapter"
    ref_dir = os.path.dirname(L.REF_SO)
    subprocess.run(["g++", "-std=c++17", "-I" + L.REF_SRC, "-I" + os.path.join(ROOT, "include"), "-o", str(exe),
                    str(d / "main.cpp"), "-L" + ref_dir, "-lref", "-L" + LIB, "-lgpuai",
                    "-Wl,-rpath," + ref_dir + ":" + LIB, "-pthread"], check=True, capture_output=True, text=True)
    return str(exe)


def test_adapter_compiles_and_converts_the_start_position(adapter_exe):
    out = subprocess.run([adapter_exe], capture_output=True, text=True, timeout=120).stdout
    assert "board 00000fff fff00000 00000000 00000000" in out


def test_adapter_reports_errors_as_exceptions(adapter_exe):
    out = subprocess.run([adapter_exe], capture_output=True, text=True, timeout=120).stdout
    if "error " in out:  # no usable GPU here: gpuai_create's status becomes an exception, not exit(1)
        assert re.search(r"error \S", out)
    else:
        assert "driver device_gb300" in out and "empty 0" in out
