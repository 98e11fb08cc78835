"""Build libbtegpu.so (CUDA kernels for sm_103a + the C ABI) and the
rtamc2d_gpu drop-in executable, in-tree under bte-barna_gb300/_build/.

Translation units compile in parallel; the replay kernels are built with
-fmad=false and all host code with -ffp-contract=off so that the replay mode
matches the CPU restatement bit for bit.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libbtegpu.so")
CLI = os.path.join(OUT, "rtamc2d_gpu")
CLI_BE = os.path.join(OUT, "bertamc2d_gpu")
CLI_DR = os.path.join(OUT, "dist_reader_gpu")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOSTFLAGS = "-fPIC,-ffp-contract=off,-O2"

UNITS = [
    # (source, extra nvcc flags)
    ("rta_replay.cu", ["-fmad=false"]),
    ("rta_prod.cu", []),
    ("capi.cu", []),
    ("noalloc.cu", []),
    ("berta.cu", []),
    ("steady.cu", []),
    ("adjoint.cu", []),
]


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(HERE), "include", "btegpu.h"))
    files.append(os.path.abspath(__file__))
    return files


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    deps = _deps()
    if (not force and _newer(LIB, deps) and _newer(CLI, deps) and _newer(CLI_BE, deps)
            and _newer(CLI_DR, deps)):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    for src, extra in UNITS:
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        jobs.append([NVCC, "-std=c++17", "-O3", "-lineinfo", *ARCH, *extra,
                     "-Xcompiler", HOSTFLAGS, "-Xptxas", "-v" if verbose else "-O3",
                     "-c", os.path.join(CSRC, src), "-o", obj])
    jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off",
                 "-I", "/usr/local/cuda/include",
                 "-c", os.path.join(CSRC, "tables.cpp"), "-o", os.path.join(OUT, "tables.o")])
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for lg in logs:
            sys.stdout.write(lg)
    objs = [os.path.join(OUT, s.replace(".cu", ".o")) for s, _ in UNITS] + [os.path.join(OUT, "tables.o")]
    tmp = LIB + ".tmp%d" % os.getpid()
    _run([NVCC, "-shared", *ARCH, "-o", tmp, *objs, "-Xcompiler", "-pthread"])
    os.replace(tmp, LIB)
    tmp = CLI + ".tmp%d" % os.getpid()
    _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", os.path.join(CSRC, "cli_rtamc2d.cpp"),
          "-o", tmp, "-L", OUT, "-lbtegpu", "-Wl,-rpath,$ORIGIN", "-pthread"])
    os.replace(tmp, CLI)
    tmp = CLI_BE + ".tmp%d" % os.getpid()
    _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", os.path.join(CSRC, "cli_bertamc2d.cpp"),
          "-o", tmp, "-L", OUT, "-lbtegpu", "-Wl,-rpath,$ORIGIN", "-pthread"])
    os.replace(tmp, CLI_BE)
    tmp = CLI_DR + ".tmp%d" % os.getpid()
    _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", os.path.join(CSRC, "cli_dist_reader.cpp"), "-o", tmp])
    os.replace(tmp, CLI_DR)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
