"""Builds liboracle.so, the CPU restatement used as the test oracle and as the
timed CPU baseline. Test infrastructure only: the product never loads it.

Portable C++ (no intrinsics; the packet traversal uses the GCC/Clang 8-float
vector extension, lowered to the target's own vector registers);
-ffp-contract=off keeps every float operation rounding where the reference's
does. On x86-64 the FMA and AVX2 instruction
sets are enabled for speed only: results are the same without them.
"""

import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
TABLES = os.path.join(os.path.dirname(HERE), "convector_gb300", "csrc")
LIB = os.path.join(HERE, "liboracle.so")
SOURCES = ["convector_oracle.cpp", "bvh_oracle.cpp", "x86sem.h"]


def build(force=False):
    srcs = [os.path.join(HERE, s) for s in SOURCES] + [os.path.join(TABLES, "x86_approx_tables.h"),
                                                      os.path.abspath(__file__)]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in srcs):
        return LIB
    flags = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-pthread"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags += ["-mfma", "-mavx2"]
    cmd = [os.environ.get("CXX", "g++")] + flags + ["-I", TABLES, "-o", LIB + ".tmp",
                                                    os.path.join(HERE, "convector_oracle.cpp"),
                                                    os.path.join(HERE, "bvh_oracle.cpp")]
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stdout)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
