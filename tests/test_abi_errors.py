"""C-ABI error behaviour without a GPU: every entry point validates its arguments on the host and
returns a negative GFGPU_ERR_* code with a message (GOOSEFEM_ASSERT's role in the reference,
config.h:140-173) instead of launching; empty inputs are no-ops."""

import ctypes as C

import numpy as np
import pytest

ERR_ARG, ERR_INDEX, ERR_UNSUPPORTED = -1, -2, -7


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__

    __graft_entry__.build()
    from goosefem_gb300 import _lib

    return _lib


@pytest.fixture(scope="module")
def L(lib):
    L = lib.lib()
    L.gfgpu_last_error.restype = C.c_char_p
    return L


def _rc(L, name, *args):
    f = getattr(L, name)
    return f(*args)


def test_null_and_empty_arguments(L):
    # null pointers
    assert _rc(L, "gfgpu_grad_n_vector", None, None, C.c_int64(4), 4, 4, 2, None, None) == ERR_ARG
    assert b"bad argument" in L.gfgpu_last_error()
    assert _rc(L, "gfgpu_quad4_compute_dN", None, C.c_int64(1), None, None, 4, None, None, None,
               None, None) == ERR_ARG
    assert _rc(L, "gfgpu_matrix_assemble", None, None, C.c_int64(1), None, None, None) == ERR_ARG
    # unsupported element types
    buf = (C.c_double * 64)()
    assert _rc(L, "gfgpu_int_grad_n_dot_tensor2_dv", buf, buf, buf, C.c_int64(1), 3, 4, 2, buf,
               None) == ERR_UNSUPPORTED
    # empty inputs are no-ops
    assert _rc(L, "gfgpu_matrix_assemble", buf, buf, C.c_int64(0), buf, buf, None) == 0
    assert _rc(L, "gfgpu_matrix_dot_dofval", buf, buf, buf, C.c_int64(0), buf, buf, None) == 0


def test_misaligned_and_oversized(L):
    raw = (C.c_double * 80)()
    mis = C.c_void_p(C.addressof(raw) + 8)  # 8-byte but not 16-byte aligned
    assert _rc(L, "gfgpu_grad_n_vector", mis, raw, C.c_int64(1), 4, 4, 2, raw, None) == ERR_ARG
    assert b"aligned" in L.gfgpu_last_error()
    big = C.c_int64(1 << 40)  # beyond the int32 tables
    assert _rc(L, "gfgpu_grad_n_vector", raw, raw, big, 4, 4, 2, raw, None) == ERR_ARG


def test_host_index_checks(L):
    conn = np.array([[0, 1, 2, 9]], dtype=np.int32)  # node 9 does not exist
    dofs = np.arange(8, dtype=np.int32).reshape(4, 2)
    total = 64
    rowptr = np.zeros(9, dtype=np.int32)
    col = np.zeros(total, dtype=np.int32)
    cptr = np.zeros(total + 1, dtype=np.int32)
    cidx = np.zeros(total, dtype=np.int32)
    nnz = C.c_int64(0)
    rc = _rc(L, "gfgpu_host_matrix_pattern", conn.ctypes.data_as(C.c_void_p),
             dofs.ctypes.data_as(C.c_void_p), C.c_int64(1), 4, C.c_int64(4), 2, C.c_int64(8),
             rowptr.ctypes.data_as(C.c_void_p), col.ctypes.data_as(C.c_void_p),
             cptr.ctypes.data_as(C.c_void_p), cidx.ctypes.data_as(C.c_void_p), C.byref(nnz))
    assert rc == ERR_INDEX and b"conn out of range" in L.gfgpu_last_error()
    ty = np.array([[0, 7]], dtype=np.int32)  # tying node beyond nnode
    ctrl = np.zeros((2, 2), dtype=np.int32)
    out_d = np.zeros_like(dofs)
    out_c = np.zeros_like(ctrl)
    counts = np.zeros(4, dtype=np.int64)
    rc = _rc(L, "gfgpu_host_tyings_periodic", dofs.ctypes.data_as(C.c_void_p), C.c_int64(4), 2,
             ctrl.ctypes.data_as(C.c_void_p), ty.ctypes.data_as(C.c_void_p), C.c_int64(1), None,
             C.c_int64(0), out_d.ctypes.data_as(C.c_void_p), out_c.ctypes.data_as(C.c_void_p),
             counts.ctypes.data_as(C.c_void_p))
    assert rc == ERR_INDEX


def test_python_layer_raises(lib):
    import goosefem_gb300 as gf

    with pytest.raises(gf.GFGPUError) as ei:
        lib.call("gfgpu_matrix_dot_dofval", None, None, None, 3, None, None, None)
    assert ei.value.code == ERR_ARG
    with pytest.raises(ValueError):
        gf.Tyings.Periodic(np.zeros((4, 2)), np.arange(8).reshape(4, 2), np.zeros((3, 3)),
                           np.array([[0, 1]]))
