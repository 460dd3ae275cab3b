"""Build libhfx.so in-tree: nvcc for the CUDA translation units
(-gencode arch=compute_103a,code=sm_103a), the host C++ compiler for the
rest, compiled in parallel and linked with nvcc (static CUDA runtime)."""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhfx.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INC = ["-I", os.path.join(REPO, "include"), "-I", CSRC, "-I", "/usr/local/cuda/include"]


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _cmd(src):
    obj = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                               "-c", path, "-o", obj] + INC
        if os.environ.get("HFX_PTXAS_VERBOSE"):
            cmd += ["-Xptxas", "-v"]
    else:
        cmd = [CXX, "-O2", "-std=c++17", "-fPIC", "-c", path, "-o", obj] + INC
    return obj, cmd


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".hpp", ".cuh"))]
    deps.append(os.path.join(REPO, "include", "hfx.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    objs = []
    for s in _sources():
        obj, cmd = _cmd(s)
        objs.append(obj)
        if force or _stale(obj, s):
            jobs.append((s, cmd))

    def run(item):
        s, cmd = item
        r = subprocess.run(cmd, capture_output=True, text=True)
        return s, r

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for s, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("compilation of %s failed" % s)
    if jobs or not os.path.exists(LIB):
        cmd = [NVCC] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", LIB] + objs + [
            "-L/usr/local/cuda/lib64", "-lcublas", "-lcusolver", "-ldl", "-lpthread",
            "-Xlinker", "-rpath", "-Xlinker", "/usr/local/cuda/lib64"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link of libhfx.so failed")
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
