"""Build recipe for oracle/_ref/libxyceref.so: the reference Xyce device code,
compiled from its own unmodified sources, plus the harness in this folder;
and oracle/_ref/libksparse.so, the reference's bundled sparse direct solver.

Test infrastructure only.  Runs where the reference source tree is present
(it is not copied into this repository); writes only under oracle/_ref/.
Usage:  python oracle/ref_build/build_ref.py [--ref /path/to/reference] [-j N]
"""
import argparse
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
REPO = os.path.dirname(os.path.dirname(HERE))
# Where the build container mounts the reference source tree (read-only).
DEFAULT_REF = "/root/reference"

OPEN_MODELS = ["MOSFET1", "MOSFET_B3", "Diode", "Resistor", "Capacitor", "Vsrc", "ISRC"]
# Core files left out: the device manager itself (replaced by the harness) and
# the reaction/TCAD machinery that needs Sacado.
CORE_SKIP = {"N_DEV_DeviceMgr", "N_DEV_RxnSet", "N_DEV_SpecieSource", "N_DEV_Region",
             "N_DEV_RegionData", "N_DEV_Reaction", "N_DEV_ReactionNetwork",
             "N_DEV_RateConstantCalculators", "N_DEV_DeviceInterface",
             "N_DEV_RegisterDevices", "N_DEV_DeviceSensitivities"}
UTIL_SKIP = {"N_UTL_FFTInterface", "N_UTL_FFTW_Interface", "N_UTL_IntelFFT_Interface",
             "N_UTL_Timer", "N_UTL_MPI", "N_UTL_ExpressionData", "N_UTL_Version"}
ERH_SKIP = {"null_streambuf", "mpi_filebuf"}


def sources(ref):
    src = os.path.join(ref, "src")
    out = [os.path.join(src, "DeviceModelPKG/OpenModels/src", f"N_DEV_{m}.C") for m in OPEN_MODELS]
    for d, skip in (("DeviceModelPKG/Core/src", CORE_SKIP), ("UtilityPKG/src", UTIL_SKIP),
                    ("ErrorHandlingPKG/src", ERH_SKIP)):
        full = os.path.join(src, d)
        for f in sorted(os.listdir(full)):
            if f.endswith(".C") and f[:-2] not in skip:
                out.append(os.path.join(full, f))
    return out


def include_dirs(ref):
    dirs = []
    for root, _, _ in os.walk(os.path.join(ref, "src")):
        if root.endswith("/include") and "/test" not in root:
            dirs.append(root)
    return sorted(dirs)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("XYCE_REFERENCE") or DEFAULT_REF,
                    help="reference source tree (default: $XYCE_REFERENCE, else the tree "
                         "this recipe was written against)")
    ap.add_argument("-j", type=int, default=os.cpu_count() or 4)
    a = ap.parse_args(argv)
    if not os.path.isdir(os.path.join(a.ref, "src", "DeviceModelPKG")):
        print(f"reference tree not found at {a.ref}; skipping", file=sys.stderr)
        return 0
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    incs = ["-I" + os.path.join(HERE, "shim"), "-I" + os.path.join(REPO, "include")]
    incs += ["-I" + d for d in include_dirs(a.ref)]
    # -ffp-contract=off: no fused multiply-add, so every product and sum is
    # rounded separately, as on the reference's x86-64 build.
    flags = ["g++", "-std=c++11", "-O2", "-fPIC", "-w", "-ffp-contract=off",
             "-include", "set", "-include", "iomanip", "-include", "cstring"]

    def compile_one(path):
        obj = os.path.join(objdir, os.path.basename(path)[:-2] + ".o")
        if os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(path):
            return obj
        r = subprocess.run(flags + incs + ["-c", path, "-o", obj], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"compile failed: {path}\n{r.stderr[-3000:]}")
        return obj

    srcs = sources(a.ref) + [os.path.join(HERE, "xref_harness.C")]
    with cf.ThreadPoolExecutor(a.j) as ex:
        objs = list(ex.map(compile_one, srcs))
    lib = os.path.join(OUT, "libxyceref.so")
    r = subprocess.run(["g++", "-shared", "-o", lib] + objs + ["-Wl,--no-undefined", "-ldl"],
                       capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("link failed\n" + r.stderr[-6000:])
    print(lib)
    print(build_tia(a.ref, a.j, incs, flags))
    print(build_ksparse(a.ref, a.j))
    return 0


# The reference's time-integration and Newton-convergence sources the
# transient pin runs (xref_tia.C), and what their objects need to link.
TIA_SOURCES = ["TimeIntegrationPKG/src/N_TIA_OneStep.C", "TimeIntegrationPKG/src/N_TIA_DataStore.C",
               "TimeIntegrationPKG/src/N_TIA_StepErrorControl.C",
               "TimeIntegrationPKG/src/N_TIA_TimeIntegrationMethods.C",
               "NonlinearSolverPKG/src/N_NLS_DampedNewton.C", "NonlinearSolverPKG/src/N_NLS_NLParams.C",
               "LoaderServicesPKG/src/N_LOA_Loader.C"]


def build_tia(ref, jobs, incs, flags):
    """oracle/_ref/libxyceref_tia.so: the reference's OneStep integrator, its
    data store's error norm and DampedNewton's convergence test, driven on
    plain arrays by xref_tia.C.  The sources are compiled with their symbols
    hidden and unused sections dropped at the link, so that only what the
    harness's entry points reach (and the vtables of the objects it builds)
    has to resolve; the device library supplies the utility and error
    packages."""
    objdir = os.path.join(OUT, "tia_obj")
    os.makedirs(objdir, exist_ok=True)
    tflags = flags + ["-ffunction-sections", "-fdata-sections", "-fvisibility=hidden"]

    def one(path):
        obj = os.path.join(objdir, os.path.basename(path)[:-2] + ".o")
        if os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(path):
            return obj
        r = subprocess.run(tflags + incs + ["-c", path, "-o", obj], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"compile failed: {path}\n{r.stderr[-3000:]}")
        return obj

    srcs = [os.path.join(ref, "src", s) for s in TIA_SOURCES] + [os.path.join(HERE, "xref_tia.C")]
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(one, srcs))
    lib = os.path.join(OUT, "libxyceref_tia.so")
    r = subprocess.run(["g++", "-shared", "-o", lib] + objs +
                       ["-L" + OUT, "-lxyceref", "-Wl,-rpath,$ORIGIN", "-Wl,--gc-sections",
                        "-Wl,--no-undefined", "-ldl"], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("TIA link failed\n" + r.stderr[-6000:])
    return lib


def build_ksparse(ref, jobs):
    """oracle/_ref/libksparse.so: the reference's bundled Kundert sparse
    direct solver (src/LinearAlgebraServicesPKG/ksparse, the KSparse option
    of its linear-solver factory), compiled from its C sources with a
    two-line Xyce_config.h.  A reference-side FP64 direct solve for the LU
    tests."""
    src = os.path.join(ref, "src", "LinearAlgebraServicesPKG", "ksparse")
    objdir = os.path.join(OUT, "ksparse_obj")
    os.makedirs(objdir, exist_ok=True)
    with open(os.path.join(objdir, "Xyce_config.h"), "w") as f:
        f.write("#include <limits.h>\n#include <float.h>\n")
    cflags = ["gcc", "-O2", "-fPIC", "-w", "-ffp-contract=off", "-I" + objdir,
              "-I" + os.path.join(src, "include")]
    cs = sorted(f for f in os.listdir(os.path.join(src, "src")) if f.endswith(".c"))

    def one(f):
        obj = os.path.join(objdir, f[:-2] + ".o")
        r = subprocess.run(cflags + ["-c", os.path.join(src, "src", f), "-o", obj],
                           capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"compile failed: {f}\n{r.stderr[-3000:]}")
        return obj

    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(one, cs))
    lib = os.path.join(OUT, "libksparse.so")
    r = subprocess.run(["gcc", "-shared", "-o", lib] + objs + ["-Wl,--no-undefined", "-lm"],
                       capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("ksparse link failed\n" + r.stderr[-4000:])
    return lib


if __name__ == "__main__":
    sys.exit(main())
