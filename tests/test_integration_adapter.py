"""The PlayoutDriver adapter a maintainer adds to the reference
(include/adapters/gpuPlayout.cpp) compiles
against the reference's own headers (src/playout.hpp:27-33,
src/state.hpp), converts the reference's States to the engine's boards (the
start position and every position of 200 random games played with the
reference's own move list), and reports a missing GPU as std::runtime_error
instead of exiting.  Runs where the reference sources are present (the build machine);
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
  // seeded random games played with the reference's own move list and
  // State::move: the adapter's board after every ply, with the move index taken
  unsigned x = 12345u;
  for (int g = 0; g < 200; g++) {
    State s = getStartingState();
    for (int ply = 0; ply < 150 && !s.isGameOver(); ply++) {
      const std::vector<Move> ms = s.getMoves();
      if (ms.empty()) break;
      x = x * 1103515245u + 12345u;
      const unsigned i = (x >> 16) % (unsigned)ms.size();
      s.move(ms[i]);
      const gpuai_board w = toBoard(s);
      std::printf("walk %d %u %08x %08x %08x %08x\n", g, i, w.p1, w.p2, w.kings, w.meta);
    }
  }
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


def test_adapter_converts_every_state_of_random_reference_games(adapter_exe):
    """Games played by the reference (State::getMoves, State::move) and
    converted by the adapter's toBoard after every ply equal the oracle's
    boards after the same moves (the oracle's move list order is the
    reference's): pieces, kings, side to move and moves since a capture."""
    out = subprocess.run([adapter_exe], capture_output=True, text=True, timeout=300).stdout
    games = {}
    for line in out.splitlines():
        if line.startswith("walk "):
            _, g, i, *words = line.split()
            games.setdefault(int(g), []).append((int(i), [int(w, 16) for w in words]))
    assert len(games) == 200
    plies = kings = captures = 0
    for steps in games.values():
        cur = L.start_board()[0]
        for i, want in steps:
            boards, moves = L.children(cur)
            cur = boards[i]
            assert [int(v) for v in cur] == want
            plies += 1
            kings += int(cur[2] != 0)
            captures += int(((int(cur[3]) >> 8) & 0xFF) == 0)
    assert plies > 10_000 and kings > 1000 and captures > 1000
