"""The allocation-free C3D8 force entry point, through the C ABI.

Callers that own all device memory themselves (their own pool, a fixed
budget) cannot let the library cudaMalloc; ftgpu_hex8_force_noalloc keeps its
scratch in a static device array instead.  This checks it against the regular
entry point (ftgpu_get_force, FP64 mode) within the FP64 parity tolerance, for
every law it accepts, on two calls in a row (the shared scratch keeps the
previous call's contents), and checks its error statuses.  The file sorts
last so that a run stopping at the first failure has already run every other
test; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import MATS

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10

ARGTYPES = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
            C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]


def node_corner_csr(conn, nNodes):
    ent = np.argsort(conn, kind="stable").astype(np.int32)  # entries e*8+corner, ascending
    cnt = np.bincount(conn, minlength=nNodes)
    ptr = np.zeros(nNodes + 1, np.int32)
    ptr[1:] = np.cumsum(cnt)
    return ptr, ent


def props9(mid):
    p = np.zeros(9)
    v = MATS.get(mid, [1000.0, 3400.0, 2.0e6])
    p[:len(v)] = v
    return p


class Case:
    """A jittered 8x6x5 block, its node -> corner map and device arrays."""

    def __init__(self):
        import torch

        import femtech_gb300 as ft
        from femtech_gb300 import meshgen as mg

        self.ft = ft
        self.L = ft.lib()
        self.L.ftgpu_hex8_force_noalloc.argtypes = ARGTYPES
        self.mesh = mg.hex_block(8, 6, 5, 0.008, 0.006, 0.005, jitter=0.1, seed=21)
        X = self.mesh["coordinates"]
        self.N, self.E = len(X), len(self.mesh["etype"])
        conn = self.mesh["connectivity"]
        ptr, ent = node_corner_csr(conn, self.N)
        dev = torch.device("cuda:0")
        self.dev = dev
        self.dX = torch.tensor(X.ravel(), dtype=torch.float64, device=dev)
        self.dconn = torch.tensor(conn, dtype=torch.int32, device=dev)
        self.dptr = torch.tensor(ptr, dtype=torch.int32, device=dev)
        self.dent = torch.tensor(ent, dtype=torch.int32, device=dev)
        self.dfi = torch.zeros(3 * self.N, dtype=torch.float64, device=dev)

    def call(self, u, mid, props, ent=None):
        import torch
        du = torch.tensor(u, dtype=torch.float64, device=self.dev)
        torch.cuda.synchronize()
        ent = self.dent if ent is None else ent
        st = self.L.ftgpu_hex8_force_noalloc(self.N, self.E, self.dX.data_ptr(),
                                             self.dconn.data_ptr(), self.dptr.data_ptr(),
                                             ent.data_ptr(), du.data_ptr(), mid,
                                             props.ctypes.data, self.dfi.data_ptr(), None)
        return st, self.dfi.cpu().numpy()


@pytest.fixture(scope="module")
def case():
    return Case()


# displacement scale per law: Ogden (6) at finite strain, the others small
@pytest.mark.parametrize("mid,scale", [(0, 2e-6), (1, 2e-6), (2, 2e-6), (3, 2e-6), (4, 2e-6),
                                       (6, 5e-5)])
def test_noalloc_force_matches_get_force_twice(case, mid, scale):
    from femtech_gb300 import meshgen as mg

    ft = case.ft
    props = props9(mid)
    mats = mg.materials([(mid, props)])
    ref = ft.Model(case.mesh, mats, precision=ft.FP64)
    rng = np.random.default_rng(5 + mid)
    for call in range(2):  # two calls in a row on the shared scratch
        u = rng.normal(0.0, scale, 3 * case.N)
        st, fi = case.call(u, mid, props)
        assert st == 0, (mid, call, st)
        fr = ref.GetForce(u)
        nr = np.linalg.norm(fr)
        if nr == 0.0:  # rigid: no stress, no force
            assert mid == 0 and not fi.any(), call
        else:
            assert np.linalg.norm(fi - fr) / nr < FP64_TOL, (mid, call)
    ref.close()


def test_noalloc_statuses(case):
    import torch

    ft = case.ft
    u = np.zeros(3 * case.N)
    # viscoelastic laws carry history between calls: rejected
    for mid in (5, 7):
        st, _ = case.call(u, mid, props9(mid))
        assert st == ft.ERR_INPUT, mid
    # unknown material ID
    assert case.call(u, 9, props9(1))[0] == ft.ERR_MATERIAL
    assert case.call(u, -1, props9(1))[0] == ft.ERR_MATERIAL
    # an inverted element: one interior node pushed through its neighbour
    X = case.mesh["coordinates"]
    inner = int(np.argmin(np.linalg.norm(X - [0.004, 0.003, 0.002], axis=1)))
    ub = np.zeros(3 * case.N)
    ub[3 * inner + 2] = -0.01
    assert case.call(ub, 1, props9(1))[0] == ft.ERR_INVERTED
    # a node -> corner entry past this call's corners is refused, not read
    bad = case.dent.clone()
    bad[7] = 8 * case.E + 3
    assert case.call(u, 1, props9(1), ent=bad)[0] == ft.ERR_INPUT
    # and the next good call is clean again
    st, fi = case.call(np.zeros(3 * case.N), 1, props9(1))
    assert st == 0 and not fi.any()
    torch.cuda.synchronize()


def test_noalloc_rejects_oversize():
    import femtech_gb300 as ft

    L = ft.lib()
    L.ftgpu_hex8_force_noalloc.argtypes = ARGTYPES
    props = np.zeros(9)
    one = C.c_void_p(1)
    st = L.ftgpu_hex8_force_noalloc(10, 32769, one, one, one, one, one, 1, props.ctypes.data,
                                    one, None)
    assert st == ft.ERR_INPUT
