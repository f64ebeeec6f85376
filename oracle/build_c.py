"""Build recipe of the C oracle (test infrastructure only): ``oracle/_ref/libes_oracle_f64.so``
(the float64 checker) and ``libes_oracle_f32.so`` (the timed CPU baseline), plain gcc + OpenMP,
portable flags only (no -march=native: the same source is built on x86_64 and aarch64)."""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(HERE, "es_oracle.c")


def lib_path(real="double"):
    return os.path.join(OUT, "libes_oracle_f64.so" if real == "double" else "libes_oracle_f32.so")


def build(force=False):
    os.makedirs(OUT, exist_ok=True)
    for real in ("double", "float"):
        out = lib_path(real)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(SRC):
            continue
        cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", f"-DREAL={real}", SRC, "-o", out, "-lm"]
        subprocess.run(cmd, check=True)
    return lib_path("double"), lib_path("float")


if __name__ == "__main__":
    print(build(force=True))
