"""Build the engine's shared libraries for sm_103a (in-tree, dsim_gb300/lib/).

  libdsim_gb300.so  native C-ABI (include/dsim.h)
  libdsim3.so       dSim3 plugin boundary (include/dsim3_abi.h)
  libdsim2.so       dSim2 plugin boundary (include/dsim2_abi.h)

Translation units are compiled in parallel with nvcc; objects are reused when
they are newer than their sources and headers.  The units holding step and
grid kernels (EXACT below) are compiled with -fmad=false, IEEE division and
square root and no flush to zero, so that each float operation rounds as in
the reference's CPU build; host code is compiled with -ffp-contract=off.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
INC = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(HERE, "lib")
OBJ = os.path.join(LIB, "obj")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
EXACT = {"mesh.cu", "cyl.cu", "accel.cu", "flat.cu", "batch.cu", "compartments.cu"}

UNITS = ["mesh.cu", "accel.cu", "flat.cu", "cyl.cu", "scan.cu", "reduce.cu", "api.cu", "compat3.cu", "compat2.cu",
         "host_formats.cpp", "noalloc.cu", "batch.cu", "serve.cpp", "compartments.cu", "simulate.cpp"]
LIBS = {
    "libdsim_gb300.so": ["api", "host_formats", "mesh", "accel", "flat", "cyl", "scan", "reduce", "noalloc", "batch", "serve", "compartments", "simulate"],
    "libdsim3.so": ["compat3", "mesh", "accel", "flat", "scan"],
    "libdsim2.so": ["compat2", "cyl", "scan"],
}


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _headers():
    hs = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit, verbose=False):
    src = os.path.join(SRC, unit)
    base = os.path.splitext(unit)[0]
    obj = os.path.join(OBJ, base + ".o")
    deps = [src] + _headers() + [os.path.abspath(__file__)]
    if not _stale(obj, deps):
        return obj, None
    cmd = [nvcc(), "-c", src, "-o", obj + ".tmp", "-O3", "-std=c++17", "-lineinfo",
           "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off", "-I", SRC, "-I", INC] + ARCH
    if unit in EXACT:
        cmd += ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        return obj, "compile %s failed:\n%s\n%s" % (unit, " ".join(cmd), p.stderr)
    os.replace(obj + ".tmp", obj)
    return obj, (p.stderr if verbose else None)


def build(verbose=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        res = list(ex.map(lambda u: _compile(u, verbose), UNITS))
    errs = [e for (_, e) in res if e and "failed" in e]
    if errs:
        raise RuntimeError("\n".join(errs))
    if verbose:
        for (_, e) in res:
            if e:
                sys.stderr.write(e)
    out = []
    for lib, parts in LIBS.items():
        target = os.path.join(LIB, lib)
        objs = [os.path.join(OBJ, p + ".o") for p in parts]
        if _stale(target, objs):
            cmd = [nvcc(), "-shared", "-o", target + ".tmp"] + objs + ARCH + ["-Xcompiler", "-fPIC", "-lpthread"]
            p = subprocess.run(cmd, capture_output=True, text=True)
            if p.returncode != 0:
                raise RuntimeError("link %s failed:\n%s\n%s" % (lib, " ".join(cmd), p.stderr))
            os.replace(target + ".tmp", target)
        out.append(target)
    return out


if __name__ == "__main__":
    for p in build(verbose="-v" in sys.argv):
        print(p)
