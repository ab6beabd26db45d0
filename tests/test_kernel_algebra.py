"""CPU checks of two algebraic rewrites the FP32 C3D8 element kernel relies on
(ft_elem.cuh, ft_materials.cuh), restated here in FP64 numpy:

* the six face areas of the characteristic length (areaHexahedronFace,
  Geometry.cpp:29-64, as called by CalculateCharacteristicLength_C3D8.cpp:6-29)
  formed from the Hadamard coefficients of the current corner coordinates, two
  opposite faces at a time (face_pair_area_max);
* the small-strain Ogden series with tr B taken from the A series through
  B = A + M + M A (mat_ogden), truncated where the host's bound says
  (upload_materials in ft_api.cu), against the eigen-decomposition form.
"""
import numpy as np
import pytest

CUBE = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                 [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
FACES = [(0, 1, 2, 3), (4, 5, 6, 7), (0, 3, 7, 4), (1, 2, 6, 5), (0, 1, 5, 4), (3, 2, 6, 7)]
# the kernel's face pairs: (a1, b1, a2, b2, aD, bD) -> c1 = h_a1 -+ h_b1, ...
PAIRS = [(0, 4, 1, 5, 3, 6), (1, 3, 2, 4, 5, 6), (0, 3, 2, 5, 4, 6)]


def corner_rule_area(xc, face):
    """areaHexahedronFace (Geometry.cpp:29-64): the parallelogram formula when
    every component of the twist vector is below 1e-6 (signed), else the 2x2
    Gauss rule of |dx/ds x dx/dt|."""
    p1, p2, p3, p4 = (xc[i] for i in face)
    cD = 0.25 * (p1 - p2 + p3 - p4)
    c1 = 0.25 * (-p1 + p2 + p3 - p4)
    c2 = 0.25 * (-p1 - p2 + p3 + p4)
    n0 = np.cross(c1, c2)
    if (cD < 1e-6).all():
        return 4 * np.linalg.norm(n0)
    n1, n2 = np.cross(cD, c2), np.cross(c1, cD)
    t = 1 / np.sqrt(3)
    return sum(np.linalg.norm(n0 + a * n1 + b * n2) for a in (-t, t) for b in (-t, t))


def hadamard(x):
    """hex_hadamard: [xi, eta, zeta, xi.eta, xi.zeta, eta.zeta, xi.eta.zeta] / 8."""
    sx = np.array([-1, 1, 1, -1, -1, 1, 1, -1], float)
    se = np.array([-1, -1, 1, 1, -1, -1, 1, 1], float)
    sz = np.array([-1, -1, -1, -1, 1, 1, 1, 1], float)
    signs = [sx, se, sz, sx * se, sx * sz, se * sz, sx * se * sz]
    return np.array([s @ x / 8 for s in signs])


def pair_areas(h, pair):
    """face_pair_area_max's two lanes: the six dot products of n0, n1, n2 and
    the four quadrature norms |n0 +- t n1 +- t n2|."""
    a1, b1, a2, b2, aD, bD = pair
    out = []
    for sg in (-1.0, 1.0):
        c1, c2, cD = h[a1] + sg * h[b1], h[a2] + sg * h[b2], h[aD] + sg * h[bD]
        n0, n1, n2 = np.cross(c1, c2), np.cross(cD, c2), np.cross(c1, cD)
        if (cD < 1e-6).all():
            out.append(4 * np.sqrt(n0 @ n0))
            continue
        t = 1 / np.sqrt(3)
        base = n0 @ n0 + (n1 @ n1 + n2 @ n2) / 3
        a01, a02, a12 = 2 * t * (n0 @ n1), 2 * t * (n0 @ n2), 2 / 3 * (n1 @ n2)
        u1, u2, v1, v2 = base + a12, base - a12, a01 + a02, a01 - a02
        out.append(sum(np.sqrt(max(v, 0.0)) for v in (u1 + v1, u1 - v1, u2 + v2, u2 - v2)))
    return out


@pytest.mark.parametrize("seed", range(3))
def test_face_pairs_match_the_corner_rule(seed):
    rng = np.random.default_rng(seed)
    worst = 0.0
    for trial in range(300):
        if trial % 10 == 0:  # a parallelepiped: every face takes the parallelogram branch
            xc = CUBE @ (np.eye(3) + rng.uniform(-0.2, 0.2, (3, 3))) * 0.01
        else:
            xc = CUBE * 0.01 + rng.uniform(-0.002, 0.002, (8, 3))
        h = hadamard(xc)
        mine = sum((pair_areas(h, p) for p in PAIRS), [])
        ref = [corner_rule_area(xc, f) for f in FACES]
        worst = max(worst, max(abs(a - b) / b for a, b in zip(mine, ref)))
    assert worst < 1e-12


def series_bound(alpha, n=9):
    """upload_materials: the largest |2E|_F (at most 0.3) at which the tail
    sum_{k > n} |binom(alpha/2 - 1, k)| (3 + 2 r) r^k stays below 1e-7 r."""
    b = [1.0]
    for k in range(n + 400):
        b.append(b[-1] * (alpha / 2 - 1 - k) / (k + 1))

    def tail(r):
        return sum(abs(b[k]) * (3 + 2 * r) * r ** k for k in range(n + 1, n + 400))

    if tail(0.3) <= 1e-7 * 0.3:
        return 0.3
    lo, hi = 0.0, 0.3
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        lo, hi = (mid, hi) if tail(mid) <= 1e-7 * mid else (lo, mid)
    return lo


def ogden_iso_series(M, alpha, n=9):
    """mat_ogden's series branch, isochoric part over c = 2 mu / alpha J^(-alpha/3):
    A - Ci - tr(B)/3 (I + Ci) with A's powers by Cayley-Hamilton and
    tr B = I1 + tr A + tr(M A)."""
    I = np.eye(3)
    I1 = np.trace(M)
    M2 = M @ M
    trM2 = np.trace(M2)
    I2 = 0.5 * (I1 * I1 - trM2)
    I3 = np.linalg.det(M)
    ser = []
    c = 1.0
    for k in range(n):
        c *= (alpha / 2 - 1 - k) / (k + 1)
        ser.append(c)
    pa, pb, pc = 0.0, 1.0, 0.0
    Aa, Ab, Ag = 0.0, ser[0], 0.0
    for k in range(1, n):
        pa, pb, pc = pc * I3, pa - pc * I2, pb + pc * I1
        Aa, Ab, Ag = Aa + ser[k] * pa, Ab + ser[k] * pb, Ag + ser[k] * pc
    trM3 = I1 * (trM2 - I2) + 3 * I3
    trB = I1 + (3 * Aa + Ab * I1 + Ag * trM2) + (Aa * I1 + Ab * trM2 + Ag * trM3)
    iC3 = 1 / (1 + I1 + I2 + I3)
    Ci = (-I3 * I - (1 + I1) * M + M2) * iC3
    A = Aa * I + Ab * M + Ag * M2
    return A - Ci - trB / 3 * (I + Ci)


def ogden_iso_eigen(M, alpha):
    """The same quantity from the eigen-decomposition of C = I + M."""
    w, V = np.linalg.eigh(np.eye(3) + M)
    Ca = V @ np.diag(w ** (alpha / 2 - 1)) @ V.T
    Cinv = V @ np.diag(1 / w) @ V.T
    return Ca - np.sum(w ** (alpha / 2)) / 3 * Cinv


@pytest.mark.parametrize("alpha", [5.0, -5.0, 0.2, 8.0, -3.0])
def test_ogden_series_with_trB_from_A_within_its_bound(alpha):
    rng = np.random.default_rng(int(abs(alpha) * 10))
    r = series_bound(alpha)
    assert r > 0.05
    worst = 0.0
    for _ in range(200):
        G = rng.normal(size=(3, 3))
        M = G + G.T
        M *= rng.uniform(0.2, 0.999) * r / np.linalg.norm(M)
        d = ogden_iso_series(M, alpha) - ogden_iso_eigen(M, alpha)
        # relative to the leading (linear) term of the stress, alpha/2 |M|
        worst = max(worst, np.linalg.norm(d) / (abs(alpha) / 2 * np.linalg.norm(M)))
    assert worst < 1e-6
