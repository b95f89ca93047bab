"""Device-array plumbing shared by the Python mirror of the GooseFEM API.

PyTorch is used only to own device memory and to hand out the current CUDA stream; every
computation runs in libgfgpu.so.
"""

import numpy as np
import torch

from . import _lib

f64 = torch.float64
i32 = torch.int32


def device():
    if not torch.cuda.is_available():
        raise RuntimeError("goosefem_gb300 needs a CUDA device (GB300, sm_103a)")
    return torch.device("cuda", torch.cuda.current_device())


def stream():
    return torch.cuda.current_stream().cuda_stream


def dev_f64(a):
    """float64 contiguous device tensor (copies numpy / host / other dtypes)."""
    if isinstance(a, torch.Tensor):
        t = a.to(device=device(), dtype=f64)
    else:
        t = torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=device())
    return t.contiguous()


def dev_i32(a):
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    a = np.asarray(a)
    if a.size and (a.min() < 0 or a.max() > np.iinfo(np.int32).max):
        raise ValueError("index table out of int32 range")
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.int32), device=device())


def host_i32(a):
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    a = np.asarray(a)
    if a.size and (a.min() < 0 or a.max() > np.iinfo(np.int32).max):
        raise ValueError("index table out of int32 range")
    return np.ascontiguousarray(a, dtype=np.int32)


def ptr(t):
    if t is None:
        return None
    if isinstance(t, np.ndarray):
        return t.ctypes.data
    return t.data_ptr()


def empty(shape, dtype=f64):
    return torch.empty(tuple(int(s) for s in shape), dtype=dtype, device=device())


def check_shape(t, shape, name):
    if tuple(t.shape) != tuple(int(s) for s in shape):
        raise ValueError(f"{name}: shape {tuple(t.shape)} != expected {tuple(shape)}")


def dof_csr(conn, dofs, ndof):
    """Dof-centric incidence CSR (host), see gfgpu_host_dof_csr."""
    conn = host_i32(conn)
    dofs = host_i32(dofs)
    nelem, nne = conn.shape
    nnode, ndim = dofs.shape
    ptr_ = np.empty(ndof + 1, dtype=np.int32)
    idx = np.empty(nelem * nne * ndim, dtype=np.int32)
    _lib.call("gfgpu_host_dof_csr", conn.ctypes.data, dofs.ctypes.data, nelem, nne, nnode, ndim,
              ndof, ptr_.ctypes.data, idx.ctypes.data)
    return ptr_, idx


def dof_csr_nodevec(dofs, ndof):
    dofs = host_i32(dofs)
    nnode, ndim = dofs.shape
    ptr_ = np.empty(ndof + 1, dtype=np.int32)
    idx = np.empty(nnode * ndim, dtype=np.int32)
    _lib.call("gfgpu_host_dof_csr_nodevec", dofs.ctypes.data, nnode, ndim, ndof, ptr_.ctypes.data,
              idx.ctypes.data)
    return ptr_, idx
