"""Compile the CPU restatement (oracle/rta_oracle.cpp) into oracle/_build/.

The oracle is test infrastructure: tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py load it; the engine never does.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libbteoracle.so")


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "rta_oracle.cpp")
    hdr = os.path.join(os.path.dirname(HERE), "include", "btegpu.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                    "-pthread", src, "-o", tmp], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
