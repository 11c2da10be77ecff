"""Build the CUDA library libmmh_gb300.so (sm_103a) in place with make + nvcc."""
import os
import subprocess
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))


def build(jobs=4, verbose=False):
    cmd = ["make", "-C", os.path.join(_HERE, "csrc"), f"-j{jobs}"]
    if not verbose:
        cmd.insert(1, "-s")
    subprocess.run(cmd, check=True)
    return os.path.join(_HERE, "_build", "libmmh_gb300.so")


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
