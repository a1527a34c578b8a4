"""Builds libxg.so (the CUDA engine) in-tree for sm_103a, and the CPU oracle.

    python -m xyce_gb300.build            # engine + oracle
The engine goes to xyce_gb300/_lib/libxg.so; objects to xyce_gb300/_build/.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libxg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FMA_SOURCES = {"lu_kernels.cu"}


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout[-4000:] + r.stderr[-8000:])
    return r


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(REPO, "include", f) for f in os.listdir(os.path.join(REPO, "include"))]
    return hs


def build_engine(verbose=False):
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    inc = ["-I" + CSRC, "-I" + os.path.join(REPO, "include")]
    heads = _headers()
    jobs = []
    # CUDA sources: load kernels twice (bit-exact and FMA), the rest once.
    cu_common = [nvcc, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
                 "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"] + ARCH + inc
    for ns, fmad in (("exact", "false"), ("fast", "true")):
        src = os.path.join(CSRC, "load_kernels.cu")
        obj = os.path.join(BUILD, f"load_kernels_{ns}.o")
        split = "1" if ns == "fast" else "0"
        jobs.append((obj, [src] + heads, cu_common + [f"-DXG_NS={ns}", f"-DXG_SPLIT_SUMS={split}",
                                                      f"-DXG_FAST_DIV={split}",
                                                      f"-fmad={fmad}", "-c", src, "-o", obj]))
    for f in sorted(os.listdir(CSRC)):
        src = os.path.join(CSRC, f)
        if f.endswith(".cu") and f != "load_kernels.cu":
            obj = os.path.join(BUILD, f[:-3] + ".o")
            # the sparse LU has no bit-parity target: contract to FMA there
            fmad = "true" if f in FMA_SOURCES else "false"
            jobs.append((obj, [src] + heads, cu_common + [f"-fmad={fmad}", "-c", src, "-o", obj]))
        elif f.endswith(".cpp"):
            obj = os.path.join(BUILD, f[:-4] + ".o")
            cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                   "-I" + os.path.join(cuda, "include")] + inc + ["-c", src, "-o", obj]
            jobs.append((obj, [src] + heads, cmd))

    def run(job):
        obj, deps, cmd = job
        if _stale(obj, deps):
            if verbose:
                print(" ".join(cmd))
            _run(cmd)
        return obj

    with cf.ThreadPoolExecutor(max(2, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(run, jobs))
    if _stale(LIB, objs):
        _run([nvcc, "-shared"] + ARCH + ["-o", LIB] + objs + ["-lcudart"])
    return LIB


ORACLE_DIR = os.path.join(REPO, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "liboracle.so")


def build_oracle():
    """The CPU oracle (test infrastructure), C compiled without contraction."""
    srcs = [os.path.join(ORACLE_DIR, f) for f in sorted(os.listdir(ORACLE_DIR)) if f.endswith(".c")]
    deps = srcs + [os.path.join(ORACLE_DIR, f) for f in os.listdir(ORACLE_DIR) if f.endswith(".h")]
    deps += [os.path.join(REPO, "include", f) for f in os.listdir(os.path.join(REPO, "include"))]
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    if _stale(ORACLE_LIB, deps):
        _run(["gcc", "-std=c11", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
              "-I" + os.path.join(REPO, "include"), "-shared", "-o", ORACLE_LIB] + srcs + ["-lm"])
    return ORACLE_LIB


ORACLE_COUNT_LIB = os.path.join(ORACLE_DIR, "_build", "liboracle_count.so")


def build_oracle_count():
    """The oracle's load compiled over a counting scalar (test
    infrastructure: algorithmic operation counts, oracle/count/)."""
    cdir = os.path.join(ORACLE_DIR, "count")
    units = ["xgo.c", "xgo_support.c", "xgo_devices.c", "xgo_bsim3.c"]
    deps = [os.path.join(ORACLE_DIR, f) for f in units] + [
        os.path.join(cdir, f) for f in os.listdir(cdir) if f.endswith((".cpp", ".hpp"))]
    deps += [os.path.join(REPO, "include", f) for f in os.listdir(os.path.join(REPO, "include"))]
    if not _stale(ORACLE_COUNT_LIB, deps):
        return ORACLE_COUNT_LIB
    os.makedirs(os.path.dirname(ORACLE_COUNT_LIB), exist_ok=True)
    objs = []
    base = ["g++", "-std=c++17", "-fpermissive", "-w", "-O2", "-fPIC", "-I" + os.path.join(REPO, "include"),
            "-I" + ORACLE_DIR]
    for u in units:
        o = os.path.join(os.path.dirname(ORACLE_COUNT_LIB), "count_" + u[:-2] + ".o")
        _run(base + [f'-DXGO_UNIT="../{u}"', "-c", os.path.join(cdir, "xgo_count_unit.cpp"), "-o", o])
        objs.append(o)
    o = os.path.join(os.path.dirname(ORACLE_COUNT_LIB), "count_main.o")
    _run(base + ["-c", os.path.join(cdir, "xgo_count.cpp"), "-o", o])
    objs.append(o)
    _run(["g++", "-shared", "-o", ORACLE_COUNT_LIB] + objs + ["-lm", "-Wl,--no-undefined"])
    return ORACLE_COUNT_LIB


if __name__ == "__main__":
    print(build_engine(verbose="-v" in sys.argv))
    print(build_oracle())
