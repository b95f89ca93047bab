"""ctypes binding of libgfgpu.so, the C ABI declared in include/gfgpu.h.

The argument and return types of every entry point are read from the header itself, so the
binding cannot drift from the declarations. Device-side calls take raw device pointers
(``tensor.data_ptr()``) and a CUDA stream handle; a failing call raises ``GFGPUError`` with the
library's message. The library is required: there is no fallback implementation.
"""

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
HEADER = os.path.join(ROOT, "include", "gfgpu.h")
LIBPATH = os.path.join(HERE, "libgfgpu.so")


class GFGPUError(RuntimeError):
    def __init__(self, name, code, msg):
        super().__init__(f"{name} failed ({code}): {msg}")
        self.code = code


class VerletDesc(C.Structure):
    """Mirror of gfgpu_verlet_desc (include/gfgpu.h)."""

    _fields_ = [
        ("nelem", C.c_int64), ("nnode", C.c_int64),
        ("nne", C.c_int32), ("ndim", C.c_int32), ("nip", C.c_int32),
        ("conn", C.c_void_p), ("dofs", C.c_void_p), ("csr_ptr", C.c_void_p), ("csr_idx", C.c_void_p),
        ("part", C.c_void_p), ("nnu", C.c_int64), ("inv", C.c_void_p),
        ("dNx", C.c_void_p), ("vol", C.c_void_p), ("K", C.c_void_p), ("G", C.c_void_p),
        ("fext", C.c_void_p), ("dt", C.c_double), ("eta", C.c_double),
        ("uniform", C.c_int32), ("hx", C.c_double), ("hy", C.c_double), ("hz", C.c_double),
        ("coef", C.c_void_p),
        ("mclass", C.c_void_p), ("mclass_inv", C.c_void_p), ("ncls", C.c_int32),
        ("reg_nx", C.c_int64), ("reg_ny", C.c_int64), ("reg_nz", C.c_int64),
        ("coef_pair", C.c_void_p), ("pair_mode", C.c_int32),
        ("pcg_pair", C.c_void_p), ("ell", C.c_void_p),
    ]


_CTYPE = {
    "int": C.c_int,
    "int32_t": C.c_int32,
    "int64_t": C.c_int64,
    "double": C.c_double,
    "float": C.c_float,
    "gfgpu_stream_t": C.c_void_p,
    "gfgpu_graph_t": C.c_void_p,
    "void": None,
}


def _parse_type(t):
    t = t.replace("const ", "").strip()
    if "*" in t:
        base = t.replace("*", "").strip()
        if base == "char":
            return C.c_char_p
        return C.c_void_p
    return _CTYPE[t]


def parse_header(path=HEADER):
    """Return {name: (restype, [argtypes])} for every prototype in include/gfgpu.h."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    protos = {}
    for m in re.finditer(r"([A-Za-z_][A-Za-z0-9_ \*]*?)\b(gfgpu_[A-Za-z0-9_]+)\s*\(([^;{]*?)\)\s*;",
                         text):
        ret, name, args = m.group(1).strip(), m.group(2), m.group(3).strip()
        if ret.startswith("typedef"):
            continue
        argtypes = []
        if args and args != "void":
            for a in args.split(","):
                a = a.strip()
                a = re.sub(r"\b[A-Za-z_][A-Za-z0-9_]*$", "", a).strip()  # drop the parameter name
                argtypes.append(_parse_type(a))
        protos[name] = (_parse_type(ret), argtypes)
    return protos


_lib = None
_protos = None


def lib():
    global _lib, _protos
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise ImportError(f"{LIBPATH} is missing: build it with `python -m goosefem_gb300.build`")
        L = C.CDLL(LIBPATH)
        _protos = parse_header()
        for name, (res, args) in _protos.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def protos():
    lib()
    return dict(_protos)


def last_error():
    return lib().gfgpu_last_error().decode()


def call(name, *args):
    """Call an int-returning entry point; raise GFGPUError on a non-zero status.

    Only entry points whose prototype was read from include/gfgpu.h are callable: without
    argtypes ctypes would pass 64-bit pointers and sizes as 32-bit ints."""
    L = lib()
    if name not in _protos:
        raise KeyError(f"{name} is not declared in {HEADER}")
    if len(args) != len(_protos[name][1]):
        raise TypeError(f"{name} takes {len(_protos[name][1])} arguments, got {len(args)}")
    f = getattr(L, name)
    rc = f(*args)
    if f.restype is C.c_int and rc != 0:
        raise GFGPUError(name, rc, last_error())
    return rc


def set_strict(flag):
    call("gfgpu_set_strict", 1 if flag else 0)
