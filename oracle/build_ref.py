#!/usr/bin/env python3
"""Build the reference's own CPU hot path into oracle/_ref/ (checker only).

TEST INFRASTRUCTURE.  This recipe compiles rfdougherty/dSim's CPU code --
dSim3/src/spinSystem.cpp (which #includes spinKernelCpu.cpp) and
dSim2/src/spinSystem.cpp -- from the sources where they lie, into two
harness executables that the golden-fixture generator
(tests/golden/make_golden.py) runs to pin the C restatement in oracle/.

Nothing here is shipped: outputs go to oracle/_ref/ (git-ignored).  The
reference tree is read-only, so the few mechanical edits are applied to a
scratch copy in oracle/_ref/src{2,3}/:

  * display-only OpenGL code is removed: the GL header include is dropped,
    every statement that is an OpenGL call is deleted, GLuint becomes an
    unsigned int and glMapBufferARB(...) becomes a null pointer.  These lines
    sit only on the useDisplay/useVbo branches, which the harnesses never take
    (no OpenGL is loaded, stubbed or run);
  * dSim3 SpinSystem::initFibers (dSim3/src/spinSystem.cpp:290-673) has no
    return statement; "return true;" is added before its closing brace;
  * dSim3 HITARRAYSIZE (spinSystem.cpp:1608, a stack buffer of 2000 hits for
    compartment assignment) is raised to 65536;
  * dSim2 spinSystem.cpp includes the unused radix-sort header
    (radixsort.cuh, never called); that include is dropped;
  * from dSim3/src/diffusion.cpp, whose main program needs OpenGL, GLUT and
    libconfig, only three pieces are taken, unchanged: the gradStruct type,
    computeTensor() and update() (oracle/_ref/src3/diffusion_parts.inc, with
    the vendored JAMA/TNT headers copied beside it).  The sequencer harness
    (refharness/seq3.cpp) defines the globals they use and stands in for the
    SpinSystem they drive;
  * from dSim2/src/diffusion.cpp, likewise, the gradStruct type, update() and
    the results-file header statements of its main() (oracle/_ref/src2/
    diffusion2_*.inc), driven by refharness/seq2.cpp.
The host side of the C-ABI (allocateArray -> malloc, copy* -> memcpy) and the
cutil timer macros are provided by oracle/refharness/.

Usage: python3 oracle/build_ref.py [--reference DIR]
"""
import argparse
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# where this recipe looks for the reference tree: DSIM_REFERENCE, else the
# checkout that this build reads (absent on machines that only run the tests)
DEFAULT_REFERENCE = "/root/reference"


def reference_dir():
    """The reference tree to build from, or None when it is not present."""
    ref = os.environ.get("DSIM_REFERENCE", DEFAULT_REFERENCE)
    return ref if os.path.isdir(ref) else None
HARNESS = os.path.join(HERE, "refharness")

DSIM3_FILES = ["spinSystem.cpp", "spinKernelCpu.cpp", "spinSystem.h", "spinSystem.cuh",
               "RTree.h", "dSimDataTypes.h"]
DSIM2_FILES = ["spinSystem.cpp", "spinKernelCpu.cpp", "spinSystem.h", "spinSystem.cuh",
               "spinKernel.cuh", "options.h"]

GL_STMT = re.compile(r"^\s*gl[A-Z]\w*\s*\(.*\)\s*;\s*(//.*)?$")
GL_REGISTER = re.compile(r"^\s*(un)?registerGLBufferObject\s*\(.*\)\s*;\s*(//.*)?$")


def strip_gl(text):
    out = []
    for line in text.split("\n"):
        if re.match(r"^\s*#include\s*<GL/", line):
            out.append("/* OpenGL include removed */")
            continue
        if GL_STMT.match(line) or GL_REGISTER.match(line):
            out.append("/* OpenGL call removed */")
            continue
        line = line.replace("glMapBufferARB(GL_ARRAY_BUFFER, GL_WRITE_ONLY)", "0")
        line = re.sub(r"\bGLuint\b", "unsigned int", line)
        out.append(line)
    return "\n".join(out)


def patch_dsim3(src):
    text = strip_gl(src)
    lines = text.split("\n")
    # initFibers ends at spinSystem.cpp:673; the loop closing braces precede it.
    idx = None
    for i, ln in enumerate(lines):
        if ln.startswith("bool SpinSystem::initFibers("):
            depth = 0
            for j in range(i, len(lines)):
                depth += lines[j].count("{") - lines[j].count("}")
                if depth == 0 and "}" in lines[j]:
                    idx = j
                    break
            break
    assert idx is not None, "initFibers not found"
    lines.insert(idx, "\treturn true; /* added: the function has no return */")
    text = "\n".join(lines)
    text, n = re.subn(r"#define HITARRAYSIZE 2000", "#define HITARRAYSIZE 65536", text)
    assert n == 1
    return text


def patch_dsim2(src):
    text = strip_gl(src)
    text, n = re.subn(r'#include "radixsort.cuh"', "/* unused radix sort header removed */", text)
    assert n == 1
    return text


def _cut(text, start):
    """The text from `start` to its matching closing brace, through the end
    of that line (a typedef's closing "} name;" included)."""
    i = text.index(start)
    depth, j, seen = 0, i, False
    while True:
        c = text[j]
        if c == "{":
            depth += 1
            seen = True
        elif c == "}":
            depth -= 1
            if seen and depth == 0:
                break
        j += 1
    k = text.index("\n", j)
    return text[i:k + 1]


def diffusion_parts(reference):
    """gradStruct, computeTensor() and update() of dSim3/src/diffusion.cpp, verbatim."""
    with open(os.path.join(reference, "dSim3", "src", "diffusion.cpp")) as fh:
        text = fh.read()
    parts = [_cut(text, "typedef struct _gradStruct{"),
             _cut(text, "void computeTensor(uint index, double tensors[][3][3]"),
             _cut(text, "void update(){")]
    return "/* taken unchanged from dSim3/src/diffusion.cpp by oracle/build_ref.py */\n" + "\n".join(parts)


def _lines_between(text, first, last):
    """The lines from the one containing `first` through the one containing
    `last`, unchanged."""
    i = text.index(first)
    i = text.rindex("\n", 0, i) + 1
    j = text.index(last, i)
    return text[i:text.index("\n", j) + 1]


def dsim2_parts(reference):
    """The gradStruct type and update() of dSim2/src/diffusion.cpp, verbatim,
    and the results-file header that its main() writes (the statements from
    the fopen of the results file through the fibers line)."""
    with open(os.path.join(reference, "dSim2", "src", "diffusion.cpp")) as fh:
        text = fh.read()
    note = "/* taken unchanged from dSim2/src/diffusion.cpp by oracle/build_ref.py */\n"
    header = _lines_between(text, 'outFilePtr = fopen(outFilename,"at");',
                            """fprintf(outFilePtr,"fibersFile{m} = '%s';\\n", fiberFileConst);""")
    return (note + _cut(text, "typedef struct _gradStruct"), note + _cut(text, "void update(){"), note + header)


def build(reference):
    os.makedirs(OUT, exist_ok=True)
    for sub in ("jama", "tnt"):
        dst = os.path.join(OUT, sub)
        if os.path.isdir(dst):
            shutil.rmtree(dst)
        shutil.copytree(os.path.join(reference, "dSim3", sub), dst)
    os.makedirs(os.path.join(OUT, "src3"), exist_ok=True)
    with open(os.path.join(OUT, "src3", "diffusion_parts.inc"), "w") as fh:
        fh.write(diffusion_parts(reference))
    os.makedirs(os.path.join(OUT, "src2"), exist_ok=True)
    for name, part in zip(("diffusion2_types.inc", "diffusion2_update.inc", "diffusion2_header.inc"),
                          dsim2_parts(reference)):
        with open(os.path.join(OUT, "src2", name), "w") as fh:
            fh.write(part)
    for tree, files, patch in (("dSim3", DSIM3_FILES, patch_dsim3),
                               ("dSim2", DSIM2_FILES, patch_dsim2)):
        dst = os.path.join(OUT, "src" + tree[-1])
        os.makedirs(dst, exist_ok=True)
        for f in files:
            shutil.copyfile(os.path.join(reference, tree, "src", f), os.path.join(dst, f))
        p = os.path.join(dst, "spinSystem.cpp")
        with open(p) as fh:
            text = fh.read()
        with open(p, "w") as fh:
            fh.write(patch(text))
    cxx = os.environ.get("CXX", "g++")
    common = [cxx, "-O2", "-ffp-contract=off", "-w", "-I", os.path.join(HARNESS, "include")]
    jobs = [
        common + ["-I", os.path.join(OUT, "src3"), os.path.join(OUT, "src3", "spinSystem.cpp"),
                  os.path.join(HARNESS, "host_abi.cpp"), os.path.join(HARNESS, "harness3.cpp"),
                  "-o", os.path.join(OUT, "harness3")],
        common + ["-I", os.path.join(OUT, "src2"), "-DDSIM2_ABI",
                  os.path.join(OUT, "src2", "spinSystem.cpp"),
                  os.path.join(HARNESS, "host_abi.cpp"), os.path.join(HARNESS, "harness2.cpp"),
                  "-o", os.path.join(OUT, "harness2")],
        common + ["-I", os.path.join(OUT, "src3"), "-I", os.path.join(OUT, "jama"), "-I", os.path.join(OUT, "tnt"),
                  os.path.join(HARNESS, "seq3.cpp"), "-o", os.path.join(OUT, "seq3")],
        common + ["-I", os.path.join(OUT, "src2"), os.path.join(HARNESS, "seq2.cpp"), "-o", os.path.join(OUT, "seq2")],
    ]
    procs = [subprocess.Popen(j) for j in jobs]
    rc = [p.wait() for p in procs]
    if any(rc):
        raise SystemExit("reference harness build failed: %r" % rc)
    return [os.path.join(OUT, "harness3"), os.path.join(OUT, "harness2")]


def sequencer_harness(dialect=3):
    """The sequencer harness that build() compiles (refharness/seq3.cpp, or
    refharness/seq2.cpp for dSim2)."""
    return os.path.join(OUT, "seq3" if dialect == 3 else "seq2")


def build_dropin(libdir):
    """The drop-in test programs: the reference's SpinSystem (the scratch copies
    in oracle/_ref/src{3,2}, prepared by build()) with its GPU branch linked
    against this project's libdsim3.so / libdsim2.so from `libdir`, in place
    of the reference's spinSystem.cu.  Built where they run (the copies travel
    with the tree; executables do not).  Returns (dropin3, dropin2) paths."""
    src3, src2 = os.path.join(OUT, "src3"), os.path.join(OUT, "src2")
    if not (os.path.exists(os.path.join(src3, "spinSystem.cpp")) and os.path.exists(os.path.join(src2, "spinSystem.cpp"))):
        raise FileNotFoundError("the reference's scratch sources are not in oracle/_ref (run build() where the "
                                "reference tree is present)")
    cxx = os.environ.get("CXX", "g++")
    # -fsigned-char: the reference's host code was written for x86-64, where char is signed
    common = [cxx, "-O2", "-ffp-contract=off", "-fsigned-char", "-w", "-I", os.path.join(HARNESS, "include")]
    rpath = ["-L", libdir, "-Wl,-rpath," + os.path.abspath(libdir)]
    out3, out2 = os.path.join(OUT, "dropin3"), os.path.join(OUT, "dropin2")
    jobs = [
        common + ["-I", src3, os.path.join(src3, "spinSystem.cpp"), os.path.join(HARNESS, "dropin3.cpp"), "-o",
                  out3] + rpath + ["-ldsim3"],
        common + ["-I", src2, "-DDSIM2_ABI", os.path.join(src2, "spinSystem.cpp"), os.path.join(HARNESS, "dropin2.cpp"),
                  "-o", out2] + rpath + ["-ldsim2"],
    ]
    procs = [subprocess.Popen(j, stderr=subprocess.PIPE) for j in jobs]
    errs = [p.communicate()[1] for p in procs]
    if any(p.returncode for p in procs):
        raise RuntimeError("drop-in build failed:\n" + "\n".join(e.decode(errors="replace")[-3000:] for e in errs))
    return out3, out2


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None, help="the reference tree (default: DSIM_REFERENCE or %s)"
                    % DEFAULT_REFERENCE)
    a = ap.parse_args()
    a.reference = a.reference or reference_dir()
    if not a.reference or not os.path.isdir(a.reference):
        print("reference tree not present; nothing to build")
        sys.exit(0)
    for p in build(a.reference):
        print(p)
