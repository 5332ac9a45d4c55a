"""Compile the C harness against include/sparc_gpu.h and link it to the
in-tree libsparc_gpu.so (gcc; no CUDA headers needed)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def build(out_dir: str) -> str:
    from sparc_gb300 import build as b
    lib = b.build()
    exe = os.path.join(out_dir, "timestepping")
    libdir = os.path.dirname(lib)
    subprocess.run(["gcc", "-O2", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "timestepping.c"), "-o", exe, "-L", libdir, "-lsparc_gpu",
                    "-Wl,-rpath," + libdir], check=True)
    return exe
