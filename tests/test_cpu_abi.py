"""The C-ABI libraries load without a GPU and export every function their
headers declare (include/dsim.h, include/dsim3_abi.h, include/dsim2_abi.h)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
HEADERS = {"dsim.h": "libdsim_gb300.so", "dsim_batch.h": "libdsim_gb300.so", "dsim_serve.h": "libdsim_gb300.so",
           "dsim_sim.h": "libdsim_gb300.so",
           "dsim3_abi.h": "libdsim3.so",
           "dsim2_abi.h": "libdsim2.so"}


def declared_functions(header):
    text = open(os.path.join(INC, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r"#[^\n]*", "", text)
    text = re.sub(r"typedef\s+struct\s*\{[^}]*\}\s*\w+\s*;", "", text, flags=re.S)
    names = re.findall(r"\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", text)
    return sorted(set(n for n in names if n not in ("if", "sizeof")))


@pytest.fixture(scope="module")
def built():
    from dsim_gb300 import build
    return build.build()


@pytest.mark.parametrize("header", sorted(HEADERS))
def test_library_exports_header(built, header):
    lib = C.CDLL(os.path.join(ROOT, "dsim_gb300", "lib", HEADERS[header]))
    names = declared_functions(header)
    assert len(names) > 5
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_reference_boundary_names_covered():
    """Every function of the reference's plugin boundary has a declaration
    (dSim3/src/spinSystem.cuh:1-59, dSim2/src/spinSystem.cuh:1-62)."""
    d3 = set(declared_functions("dsim3_abi.h"))
    for n in ["checkCUDA", "allocateArray", "freeArray", "threadSync", "copyArrayFromDevice",
              "copyArrayToDevice", "registerGLBufferObject", "unregisterGLBufferObject",
              "copyConstantToDevice", "bindCubeCounter", "unbindCubeCounter", "bindTrianglesInCubes",
              "unbindTrianglesInCubes", "bindVertices", "unbindVertices", "bindTriangleHelpers",
              "unbindTriangleHelpers", "bindRTreeArray", "unbindRTreeArray", "bindTreeIndexArray",
              "unbindTreeIndexArray", "bindTriInfo", "unbindTriInfo", "integrateSystem",
              "integrateSystemVBO"]:
        assert n in d3, n
    d2 = set(declared_functions("dsim2_abi.h"))
    for n in ["checkCUDA", "allocateArray", "freeArray", "threadSync", "copyArrayFromDevice",
              "copyArrayToDevice", "registerGLBufferObject", "unregisterGLBufferObject",
              "bindFiberList", "unbindFiberList", "bindCubeList", "unbindCubeList",
              "integrateSystem", "integrateSystemVbo"]:
        assert n in d2, n


def test_python_binding_declares_every_native_symbol(built):
    from dsim_gb300 import _lib
    L = _lib.native()
    for n in declared_functions("dsim.h"):
        assert getattr(L, n).argtypes is not None or getattr(L, n).restype is not None, n
