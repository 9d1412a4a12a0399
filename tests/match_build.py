"""Builds tests/_build/match (the GPU-vs-mcts_host match, test infrastructure)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build", "match")


def build_match() -> str:
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    obj = os.path.join(HERE, "_build", "oracle_match.o")
    subprocess.run(["gcc", "-O2", "-fopenmp", "-std=c11", "-c", os.path.join(ROOT, "oracle", "oracle.c"), "-o", obj],
                   check=True)
    lib = os.path.join(ROOT, "gpu_ai_gb300", "lib")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fopenmp", "-pthread", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(ROOT, "gpu_ai_gb300", "csrc"), "-o", OUT,
                    os.path.join(HERE, "match.cpp"), obj, "-L" + lib, "-lgpuai", "-Wl,-rpath," + lib], check=True)
    return OUT


if __name__ == "__main__":
    print(build_match())
