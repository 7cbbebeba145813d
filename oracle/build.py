"""Build recipe of the oracle (test infrastructure; see nemo_oracle.h).

gcc -O3 -ffp-contract=off -fno-fast-math: no multiply-add fusion and no
reassociation, so each FP64 operation rounds like the reference's gfortran build
without FMA contraction (-O3's vectorisation keeps every operation and its order).
No -march/-mcpu=native: the same source builds on the x86 container and on the
Arm host of the GPU and must give the same results on both.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "libnemo_oracle.so")


def build(force=False):
    src = os.path.join(HERE, "nemo_oracle.c")
    hdrs = [os.path.join(HERE, "nemo_oracle.h"), os.path.join(os.path.dirname(HERE), "include", "nemo_gpu.h")]
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if not force and os.path.exists(OUT) and all(os.path.getmtime(p) < os.path.getmtime(OUT) for p in [src] + hdrs):
        return OUT
    cmd = ["gcc", "-std=c11", "-O3", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-fPIC", "-shared",
           "-fopenmp", "-o", OUT, src, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
