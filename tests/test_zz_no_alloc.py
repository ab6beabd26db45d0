"""The allocation-free C3D8 force entry point, through the C ABI.

Callers that own all device memory themselves (their own pool, a fixed
budget) cannot let the library cudaMalloc; ftgpu_hex8_force_noalloc keeps its
scratch in a static device array instead.  This checks it against the regular
entry point (ftgpu_get_force, FP64 mode) within the FP64 parity tolerance, on
two calls in a row (the shared scratch keeps the previous call's contents).
The file sorts last so that a run stopping at the first failure has already
run every other test; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def node_corner_csr(conn, nNodes):
    ent = np.argsort(conn, kind="stable").astype(np.int32)  # entries e*8+corner, ascending
    cnt = np.bincount(conn, minlength=nNodes)
    ptr = np.zeros(nNodes + 1, np.int32)
    ptr[1:] = np.cumsum(cnt)
    return ptr, ent


def test_noalloc_force_matches_get_force_twice():
    import torch

    import femtech_gb300 as ft
    from femtech_gb300 import meshgen as mg

    L = ft.lib()
    L.ftgpu_hex8_force_noalloc.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
    mesh = mg.hex_block(8, 6, 5, 0.008, 0.006, 0.005, jitter=0.1, seed=21)
    props = np.array([1000.0, 3400.0, 2.0e6, 0, 0, 0, 0, 0, 0])
    mats = mg.materials([(1, props[:3])])
    X = mesh["coordinates"]
    N, E = len(X), len(mesh["etype"])
    conn = mesh["connectivity"]
    ptr, ent = node_corner_csr(conn, N)
    dev = torch.device("cuda:0")
    dX = torch.tensor(X.ravel(), dtype=torch.float64, device=dev)
    dconn = torch.tensor(conn, dtype=torch.int32, device=dev)
    dptr = torch.tensor(ptr, dtype=torch.int32, device=dev)
    dent = torch.tensor(ent, dtype=torch.int32, device=dev)
    dfi = torch.zeros(3 * N, dtype=torch.float64, device=dev)
    ref = ft.Model(mesh, mats, precision=ft.FP64)
    rng = np.random.default_rng(5)
    for call in range(2):  # two calls in a row on the shared scratch
        u = rng.normal(0.0, 2e-6, 3 * N)
        du = torch.tensor(u, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        st = L.ftgpu_hex8_force_noalloc(N, E, dX.data_ptr(), dconn.data_ptr(), dptr.data_ptr(),
                                        dent.data_ptr(), du.data_ptr(), 1, props.ctypes.data,
                                        dfi.data_ptr(), None)
        assert st == 0, (call, st)
        fi = dfi.cpu().numpy()
        fr = ref.GetForce(u)
        assert np.linalg.norm(fi - fr) / np.linalg.norm(fr) < FP64_TOL, call
    ref.close()


def test_noalloc_rejects_oversize():
    import femtech_gb300 as ft

    L = ft.lib()
    L.ftgpu_hex8_force_noalloc.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
    props = np.zeros(9)
    one = C.c_void_p(1)
    st = L.ftgpu_hex8_force_noalloc(10, 32769, one, one, one, one, one, 1, props.ctypes.data,
                                    one, None)
    assert st == ft.ERR_INPUT
