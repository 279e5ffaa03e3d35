"""Build recipe of libsu2gpu.so (in-tree, next to this file).

The kernels are instantiated per precision (FP64 plain path, FP32 precision
form) and per field content (a specialisation for the fundamental, adjoint and
SU(2)xU(1)+singlet contents, plus a generic one that reads the content at run
time); the units compile in parallel.  Only sm_103a is targeted.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsu2gpu.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", ARCH, "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Wno-deprecated-gpu-targets", "--expt-relaxed-constexpr"]

# FP32 units: approximate division and square root, denormals flushed (the
# FP32 form is validated statistically; the FP64 units keep IEEE arithmetic)
FP32_FLAGS = ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"]

UNITS = [
    # name, source, defines
    ("inst_f64_generic", "su2_inst.cu", ["SU2_R=double", "SU2_CC=-1", "SU2_OPS=ops_f64_generic",
                                          "SU2_WITH_PREC=precops_f64", "SU2_WITH_GLOBAL"]),
    ("inst_f64_fund", "su2_inst.cu", ["SU2_R=double", "SU2_CC=1", "SU2_OPS=ops_f64_fund"]),
    ("inst_f64_adj", "su2_inst.cu", ["SU2_R=double", "SU2_CC=4", "SU2_OPS=ops_f64_adj"]),
    ("inst_f64_su2u1s", "su2_inst.cu", ["SU2_R=double", "SU2_CC=25", "SU2_OPS=ops_f64_su2u1s"]),
    ("inst_f32_generic", "su2_inst.cu", ["SU2_R=float", "SU2_CC=-1", "SU2_OPS=ops_f32_generic",
                                          "SU2_WITH_PREC=precops_f32"]),
    ("inst_f32_fund", "su2_inst.cu", ["SU2_R=float", "SU2_CC=1", "SU2_OPS=ops_f32_fund"]),
    ("inst_f32_adj", "su2_inst.cu", ["SU2_R=float", "SU2_CC=4", "SU2_OPS=ops_f32_adj"]),
    ("inst_f32_su2u1s", "su2_inst.cu", ["SU2_R=float", "SU2_CC=25", "SU2_OPS=ops_f32_su2u1s"]),
    ("persist_f64_generic", "su2_persist.cu", ["SU2_R=double", "SU2_CC=-1", "SU2_PERSIST=persist_f64_generic"]),
    ("persist_f64_fund", "su2_persist.cu", ["SU2_R=double", "SU2_CC=1", "SU2_PERSIST=persist_f64_fund"]),
    ("persist_f64_adj", "su2_persist.cu", ["SU2_R=double", "SU2_CC=4", "SU2_PERSIST=persist_f64_adj"]),
    ("persist_f64_su2u1s", "su2_persist.cu", ["SU2_R=double", "SU2_CC=25", "SU2_PERSIST=persist_f64_su2u1s"]),
    ("persist_f32_generic", "su2_persist.cu", ["SU2_R=float", "SU2_CC=-1", "SU2_PERSIST=persist_f32_generic"]),
    ("persist_f32_fund", "su2_persist.cu", ["SU2_R=float", "SU2_CC=1", "SU2_PERSIST=persist_f32_fund"]),
    ("persist_f32_adj", "su2_persist.cu", ["SU2_R=float", "SU2_CC=4", "SU2_PERSIST=persist_f32_adj"]),
    ("persist_f32_su2u1s", "su2_persist.cu", ["SU2_R=float", "SU2_CC=25", "SU2_PERSIST=persist_f32_su2u1s"]),
    ("su2gpu", "su2gpu.cu", []),
    ("su2_noalloc", "su2_noalloc.cu", []),
    ("su2_pool", "su2_pool.cu", []),
    ("su2_correl", "su2_correl.cu", []),
    ("su2_probe", "su2_probe.cu", []),
]
EXTRA_SOURCES = []  # (name, source) of further host units, appended by later modules


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsu2gpu")


def _sources():
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    out.append(os.path.join(os.path.dirname(HERE), "include", "su2gpu.h"))
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, force=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()
    deps = _sources()
    units = list(UNITS)
    for name, src in EXTRA_SOURCES:
        units.append((name, src, []))

    def compile_unit(u):
        name, src, defs = u
        obj = os.path.join(BUILD, name + ".o")
        if not force and not _stale(obj, deps):
            return obj
        # the allocation-free unit instantiates FP32 kernels too: same FP32 flags
        # (they change single-precision arithmetic only)
        extra = FP32_FLAGS if ("SU2_R=float" in defs or name == "su2_noalloc") else []
        cmd = [exe] + NVCC_FLAGS + extra + ["-D" + d for d in defs] + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(units), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_unit, units))
    if force or _stale(LIB, objs):
        cmd = [exe, ARCH, "-shared", "-cudart=static", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
