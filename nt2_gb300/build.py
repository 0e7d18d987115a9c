"""In-tree builds: libnt2gpu.so (nvcc, sm_103a) and the C++ table-layer
examples.  Nothing is installed; outputs go to nt2_gb300/_build/."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def build_library(jobs=None):
    jobs = jobs or max(2, min(8, os.cpu_count() or 2))
    subprocess.run(["make", "-C", HERE, f"-j{jobs}"], check=True)
    return os.path.join(HERE, "_build", "libnt2gpu.so")
