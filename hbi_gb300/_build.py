"""In-tree build of libhbigpu.so (sm_103a) -- nvcc + g++, no cmake.

The host translation units are compiled with -ffp-contract=off so the
cluster tree / admissibility arithmetic gives the same bits on x86_64 and
aarch64 (and the same bits as the CPU oracle).
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libhbigpu.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I" + CSRC]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-I" + CSRC]

CU = ["hbi_capi.cu", "hbi_aca.cu", "hbi_aca_okada.cu", "hbi_aca_td.cu", "hbi_aca_tdhs.cu", "hbi_matvec.cu", "hbi_stream.cu", "hbi_cycle.cu", "hbi_mlp.cu", "hbi_umma_probe.cu", "hbi_ens.cu", "hbi_enstc.cu"]
CPP = ["hbi_structure.cpp"]


def _sources():
    cu = [s for s in CU if os.path.exists(os.path.join(CSRC, s))]
    return cu, CPP


def _newer(src_list, target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in src_list)


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    cu, cpp = _sources()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".hpp", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "hbi_gpu.h"))
    jobs, objs = [], []
    for s in cu:
        o = os.path.join(OBJ, s + ".o")
        objs.append(o)
        if force or _newer([os.path.join(CSRC, s)] + headers, o):
            jobs.append([NVCC] + ARCH + NVFLAGS + ["-c", os.path.join(CSRC, s), "-o", o])
    for s in cpp:
        o = os.path.join(OBJ, s + ".o")
        objs.append(o)
        if force or _newer([os.path.join(CSRC, s)] + headers, o):
            jobs.append(["g++"] + CXXFLAGS + ["-c", os.path.join(CSRC, s), "-o", o])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for out in ex.map(_compile, jobs):
            if verbose and out.strip():
                print(out, file=sys.stderr)
    if force or jobs or _newer(objs, LIB):
        _compile([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
