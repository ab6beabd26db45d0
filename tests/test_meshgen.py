"""Synthetic workload generators: sizes, orientation and load sets."""
import numpy as np

from femtech_gb300 import meshgen as mg


def hex_volumes(mesh):
    X = mesh["coordinates"]
    c = mesh["connectivity"].reshape(-1, 8)
    a, b, d, e = X[c[:, 0]], X[c[:, 1]], X[c[:, 3]], X[c[:, 4]]
    return np.einsum("ij,ij->i", np.cross(b - a, d - a), e - a)


def test_hex_block_counts_and_orientation():
    m = mg.hex_block(4, 3, 2, 0.4, 0.3, 0.2, jitter=0.1, seed=3)
    assert len(m["coordinates"]) == 5 * 4 * 3
    assert len(m["etype"]) == 24
    assert np.all(hex_volumes(m) > 0)
    # faces stay planar under tangential jitter
    X = m["coordinates"]
    assert np.sum(np.abs(X[:, 2]) < 1e-12) == 5 * 4


def test_scale_block_shape_is_4m_elements():
    nx, ny, nz = 200, 200, 100
    assert nx * ny * nz == 4_000_000 and (nx + 1) * (ny + 1) * (nz + 1) == 4_080_501


def test_tet_ellipsoid_positive_volumes():
    m = mg.tet_ellipsoid(0.01, 0.008, 0.007, 0.002, seed=1)
    X = m["coordinates"]
    T = m["connectivity"].reshape(-1, 4)
    v = np.einsum("ij,ij->i", np.cross(X[T[:, 0]] - X[T[:, 3]], X[T[:, 1]] - X[T[:, 3]]),
                  X[T[:, 2]] - X[T[:, 3]])
    assert np.all(v > 0) and len(T) > 100


def test_loads_tables():
    mesh, mats, loads = mg.cube_tension_case(n=2)
    assert loads.boundary.sum() == 9 * 3 + 9
    assert loads.fns[1][0] == mg.BCK_RAMP
