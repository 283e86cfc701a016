"""In-tree build of libleo2d_gb300.so (CUDA for sm_103a + C++ host code) and
of the `leo2d` driver executable.

    python -m leo2d_gb300.build        # or __graft_entry__.build()

Translation units are compiled in parallel with nvcc / g++ and linked with
nvcc into leo2d_gb300/lib/. No CMake, no torch extension machinery.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OBJ = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(HERE, "lib", "libleo2d_gb300.so")
BIN = os.path.join(HERE, "bin", "leo2d")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-ffp-contract=off", "--expt-relaxed-constexpr", "-I" + REPO]
# files whose FP64 arithmetic must follow the reference without fused multiply-add
NO_FMAD = {"geom.cu"}
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + REPO]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(HOST) if f.endswith(".cpp") and f != "main.cpp")
    return cu, cpp


def _newer(src_list, target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in src_list)


def build(force=False, verbose=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    cu, cpp = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")]
    headers += [os.path.join(REPO, "include", f) for f in os.listdir(os.path.join(REPO, "include"))]
    tasks = []
    objs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJ, f[:-3] + ".o")
        objs.append(obj)
        if force or _newer([src] + headers, obj):
            flags = list(NVCC_FLAGS) + (["-fmad=false"] if f in NO_FMAD else [])
            tasks.append([nvcc()] + ARCH + flags + ["-c", src, "-o", obj])
    for f in cpp:
        src = os.path.join(HOST, f)
        obj = os.path.join(OBJ, "host_" + f[:-4] + ".o")
        objs.append(obj)
        if force or _newer([src] + headers, obj):
            tasks.append(["g++"] + CXX_FLAGS + ["-I" + os.path.join(_cuda_home(), "include"),
                                                "-c", src, "-o", obj])
    jobs = jobs or min(len(tasks) or 1, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for out in ex.map(_run, tasks):
            if verbose and out.strip():
                print(out)
    if force or tasks or not os.path.exists(LIB):
        _run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    main_src = os.path.join(HOST, "main.cpp")
    if os.path.exists(main_src) and (force or _newer([main_src, LIB] + headers, BIN)):
        _run(["g++"] + CXX_FLAGS + ["-o", BIN, main_src, "-L" + os.path.dirname(LIB),
                                    "-lleo2d_gb300", "-Wl,-rpath,$ORIGIN/../lib"])
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
