"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/gb_oracle.c into oracle/_build/libgb_oracle.so with gcc.
-ffp-contract=off plus explicit fma() calls make the oracle's results
bit-identical on x86-64 and aarch64; on x86-64 -mfma lets gcc emit the
hardware instruction for those fma() calls instead of a libm call.
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgb_oracle.so")
SRC = os.path.join(HERE, "gb_oracle.c")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                             os.path.getmtime(os.path.join(HERE, "gb_oracle.h")))):
        return LIB
    flags = ["-O3", "-std=gnu11", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
             "-fno-math-errno"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags += ["-mfma", "-mavx2"]
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc"] + flags + [SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
