"""Seeded synthetic meshes and load cases in FemTech's array layout.

The reference reads LS-DYNA/Abaqus decks into ``coordinates[3*nNodes]``,
``eptr``/``connectivity`` (CSR), ``ElementType`` and ``pid``
(src/io/input/ReadLsDyna.cpp, ReadAbaqus.cpp).  The benchmark workloads here
are synthetic, so these helpers build the same arrays directly:

* ``hex_block``      structured C3D8 block, optional seeded node jitter;
* ``tet_ellipsoid``  C3D4 ellipsoid from a jittered lattice + Delaunay;
* ``Loads``          per-DOF boundary-condition table (fixed / ramp / sine /
                     rigid rotation) in the form the C ABI takes.

Node order of a C3D8 element follows the reference's convention (bottom face
counter-clockwise, then top face; ShapeFunction_C3D8.cpp:26-33).
"""
import numpy as np

C3D8, C3D4 = 0, 1
BC_FREE, BC_HOLD = -1, -2
BCK_FIXED, BCK_RAMP, BCK_SINE, BCK_ROT, BCK_RIGID = 0, 1, 2, 3, 4


def hex_block(nx, ny, nz, lx, ly, lz, jitter=0.0, seed=0, origin=(0.0, 0.0, 0.0)):
    """Structured nx*ny*nz C3D8 block of size lx*ly*lz.

    ``jitter`` is the uniform node perturbation as a fraction of the local edge
    length.  Interior nodes move in all directions; nodes on a face move only
    tangentially, so the six faces stay planar and coordinate-selected
    boundary sets are unchanged.
    """
    hx, hy, hz = lx / nx, ly / ny, lz / nz
    i = np.arange(nx + 1)
    j = np.arange(ny + 1)
    k = np.arange(nz + 1)
    K, J, I = np.meshgrid(k, j, i, indexing="ij")
    X = np.stack([origin[0] + I * hx, origin[1] + J * hy, origin[2] + K * hz], -1).reshape(-1, 3)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter, jitter, size=X.shape) * np.array([hx, hy, hz])
        Ii, Jj, Kk = I.ravel(), J.ravel(), K.ravel()
        d[(Ii == 0) | (Ii == nx), 0] = 0.0
        d[(Jj == 0) | (Jj == ny), 1] = 0.0
        d[(Kk == 0) | (Kk == nz), 2] = 0.0
        X = X + d
    # element ordering: i fastest, then j, then k
    kk, jj, ii = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ii, jj, kk = ii.ravel(), jj.ravel(), kk.ravel()

    def nid(a, b, c):
        return a + (nx + 1) * (b + (ny + 1) * c)

    conn = np.stack([nid(ii, jj, kk), nid(ii + 1, jj, kk), nid(ii + 1, jj + 1, kk),
                     nid(ii, jj + 1, kk), nid(ii, jj, kk + 1), nid(ii + 1, jj, kk + 1),
                     nid(ii + 1, jj + 1, kk + 1), nid(ii, jj + 1, kk + 1)], -1)
    E = conn.shape[0]
    return dict(coordinates=np.ascontiguousarray(X, np.float64),
                eptr=np.arange(0, 8 * E + 1, 8, dtype=np.int32),
                connectivity=conn.astype(np.int32).ravel(),
                etype=np.full(E, C3D8, np.int32), pid=np.zeros(E, np.int32),
                shape=(nx, ny, nz), h=(hx, hy, hz))


def tet_ellipsoid(a, b, c, h, jitter=0.1, seed=0):
    """C3D4 mesh of the ellipsoid x^2/a^2 + y^2/b^2 + z^2/c^2 <= 1.

    Lattice of spacing h; every lattice cube whose centre lies inside is split
    into the 6 tetrahedra of its Kuhn (Freudenthal) subdivision -- the
    Delaunay triangulation of the lattice with a consistent diagonal, so the
    mesh is conforming and free of slivers -- then all nodes are jittered by
    +-jitter*h (seeded).  The surface is the resulting staircase.  Node order
    is made right-handed (positive signed volume).
    """
    rng = np.random.default_rng(seed)
    nx, ny, nz = (int(np.ceil(2 * s / h)) + 1 for s in (a, b, c))
    o = np.array([-a, -b, -c]) - 0.5 * (np.array([nx, ny, nz]) * h - 2 * np.array([a, b, c]))
    ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    cen = o + (np.stack([ci, cj, ck], -1).reshape(-1, 3) + 0.5) * h
    ins = (cen[:, 0] / a) ** 2 + (cen[:, 1] / b) ** 2 + (cen[:, 2] / c) ** 2 < 1.0
    cubes = np.stack([ci.ravel(), cj.ravel(), ck.ravel()], -1)[ins]

    def nid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)

    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    tets = []
    for p in perms:
        path = [np.zeros(3, np.int64)]
        for ax in p:
            step = path[-1].copy()
            step[ax] += 1
            path.append(step)
        tets.append(np.stack([nid(cubes[:, 0] + q[0], cubes[:, 1] + q[1], cubes[:, 2] + q[2])
                              for q in path], -1))
    T = np.concatenate(tets, 0)
    gi, gj, gk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    X = o + np.stack([gi.transpose(2, 1, 0).ravel(), gj.transpose(2, 1, 0).ravel(),
                      gk.transpose(2, 1, 0).ravel()], -1) * h
    X = X + rng.uniform(-jitter, jitter, X.shape) * h
    v = np.einsum("ij,ij->i", np.cross(X[T[:, 0]] - X[T[:, 3]], X[T[:, 1]] - X[T[:, 3]]),
                  X[T[:, 2]] - X[T[:, 3]])
    neg = v < 0
    T[neg, 0], T[neg, 1] = T[neg, 1].copy(), T[neg, 0].copy()
    used = np.unique(T)
    remap = -np.ones(len(X), np.int64)
    remap[used] = np.arange(len(used))
    T = remap[T]
    X = X[used]
    E = len(T)
    return dict(coordinates=np.ascontiguousarray(X, np.float64),
                eptr=np.arange(0, 4 * E + 1, 4, dtype=np.int32),
                connectivity=T.astype(np.int32).ravel(), etype=np.full(E, C3D4, np.int32),
                pid=np.zeros(E, np.int32))


def materials(parts):
    """parts: list of (materialID, [props...]) -> dict(materialID, properties[9*nPID])."""
    mid = np.array([p[0] for p in parts], np.int32)
    pr = np.zeros((len(parts), 9))
    for i, (_, props) in enumerate(parts):
        pr[i, : len(props)] = props
    return dict(materialID=mid, properties=pr.ravel())


class Loads:
    """Per-DOF boundary functions: -1 free, -2 hold, >= 0 index into ``fns``."""

    def __init__(self, nNodes):
        self.dof_fn = np.full(3 * nNodes, BC_FREE, np.int32)
        self.fns = []

    def add_fn(self, kind, params):
        self.fns.append((int(kind), [float(p) for p in params]))
        return len(self.fns) - 1

    def fix(self, nodes, dofs=(0, 1, 2), value=0.0):
        f = self.add_fn(BCK_FIXED, [value])
        for d in dofs:
            self.dof_fn[3 * np.asarray(nodes) + d] = f
        return f

    def ramp(self, nodes, dof, rate):
        f = self.add_fn(BCK_RAMP, [rate])
        self.dof_fn[3 * np.asarray(nodes) + dof] = f
        return f

    def sine(self, nodes, dof, amplitude, omega):
        f = self.add_fn(BCK_SINE, [amplitude, omega])
        self.dof_fn[3 * np.asarray(nodes) + dof] = f
        return f

    def rotation(self, nodes, axis, center, alpha_peak, duration):
        ax = np.asarray(axis, np.float64)
        ax = ax / np.linalg.norm(ax)
        f = self.add_fn(BCK_ROT, list(ax) + list(center) + [alpha_peak, duration])
        for d in range(3):
            self.dof_fn[3 * np.asarray(nodes) + d] = f
        return f

    def rigid(self, nodes):
        """All DOFs of ``nodes`` follow their instance's rigid body (acceleration
        records given to Model.set_rigid_body)."""
        f = self.add_fn(BCK_RIGID, [])
        for d in range(3):
            self.dof_fn[3 * np.asarray(nodes) + d] = f
        return f

    def hold(self, nodes, dofs=(0, 1, 2)):
        for d in dofs:
            self.dof_fn[3 * np.asarray(nodes) + d] = BC_HOLD

    @property
    def boundary(self):
        return (self.dof_fn != BC_FREE).astype(np.int32)


def cube_tension_case(n=10, size=0.01, rho=1000.0, mu=3400.0, K=2.0e6, strain=0.1,
                      t_ramp=0.01):
    """Unit-cube tension: n^3 C3D8 cube, z=0 face fixed, top face pulled in z,
    displacement ramped linearly to ``strain`` over ``t_ramp`` (the plain,
    CPU-runnable configuration: 10x10x10, 0.01 m, Neo-Hookean)."""
    mesh = hex_block(n, n, n, size, size, size)
    lam = K - 2.0 * mu / 3.0
    mats = materials([(1, [rho, mu, lam])])
    X = mesh["coordinates"]
    tol = 1e-9
    loads = Loads(len(X))
    loads.fix(np.where(np.abs(X[:, 2]) < tol)[0])
    loads.ramp(np.where(np.abs(X[:, 2] - size) < tol)[0], 2, strain * size / t_ramp)
    return mesh, mats, loads


def boundary_nodes_tet(conn):
    """Nodes on the boundary of a C3D4 mesh (faces used by exactly one tet)."""
    T = np.asarray(conn).reshape(-1, 4)
    faces = np.concatenate([T[:, [1, 2, 3]], T[:, [0, 2, 3]], T[:, [0, 1, 3]], T[:, [0, 1, 2]]])
    faces = np.sort(faces, axis=1)
    uniq, cnt = np.unique(faces, axis=0, return_counts=True)
    return np.unique(uniq[cnt == 1])


def smooth_fibers(X, seed=0, modes=6, scale=0.05):
    """Unit fibre directions from a seeded smooth random field: a sum of a few
    random Fourier modes per component, normalised."""
    rng = np.random.default_rng(seed)
    a = np.zeros_like(X)
    for _ in range(modes):
        k = rng.normal(0.0, 1.0 / scale, 3)
        ph = rng.uniform(0, 2 * np.pi, 3)
        amp = rng.normal(0.0, 1.0, 3)
        a += amp * np.sin(X @ k[:, None] + ph)
    n = np.linalg.norm(a, axis=1, keepdims=True)
    a[n[:, 0] < 1e-12] = [1.0, 0.0, 0.0]
    return a / np.maximum(np.linalg.norm(a, axis=1, keepdims=True), 1e-12)


def head_case(a=0.09, b=0.07, c=0.06, h=None, target_elements=2_000_000, shell=0.005, seed=0,
              E_shell=6.0e9, nu_shell=0.3, rho_shell=2000.0, mu=1.0e3, k1=5.0e3, k2=10.0,
              kappa=0.1, lam=2.19e8, rho=1040.0, g1=0.6, tau1=6.0e-3, alpha_peak=6.0e3,
              pulse=0.01):
    """Head-like C3D4 ellipsoid: outer `shell` layer Neo-Hookean (E, nu given),
    interior anisotropic GOH (fibre field, dispersion kappa) + 1-term Prony;
    boundary nodes follow a rigid rotation about a seeded random axis with
    angular acceleration alpha_peak sin(pi t / pulse) for t <= pulse."""
    if h is None:  # 6 tets per lattice cube inside the ellipsoid volume
        vol = 4.0 / 3.0 * np.pi * a * b * c
        h = (vol * 6.0 / target_elements) ** (1.0 / 3.0)
    mesh = tet_ellipsoid(a, b, c, h, jitter=0.1, seed=seed)
    X = mesh["coordinates"]
    T = mesh["connectivity"].reshape(-1, 4)
    cen = X[T].mean(1)
    rho_s = np.sqrt((cen[:, 0] / a) ** 2 + (cen[:, 1] / b) ** 2 + (cen[:, 2] / c) ** 2)
    depth = np.linalg.norm(cen, axis=1) * (1.0 / np.maximum(rho_s, 1e-9) - 1.0)
    in_shell = depth < shell
    mesh["pid"] = np.where(in_shell, 0, 1).astype(np.int32)
    mesh["fiber"] = smooth_fibers(cen, seed=seed + 1)
    mu_s = E_shell / (2 * (1 + nu_shell))
    lam_s = E_shell * nu_shell / ((1 + nu_shell) * (1 - 2 * nu_shell))
    mats = materials([(1, [rho_shell, mu_s, lam_s]),
                      (7, [rho, mu, lam, k1, k2, g1, tau1, kappa])])
    rng = np.random.default_rng(seed + 2)
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    loads = Loads(len(X))
    loads.rotation(boundary_nodes_tet(mesh["connectivity"]), axis, [0.0, 0.0, 0.0], alpha_peak,
                   pulse)
    return mesh, mats, loads


def rigid_nodes(mesh, mats):
    """Nodes of the elements whose part has material 0 (rigid), sorted and
    unique: the node set the brain drivers give the rigid-body motion
    (examples/ex5/ex5.cpp:809-840)."""
    mid = np.asarray(mats["materialID"])
    pid = np.asarray(mesh["pid"])
    eptr = np.asarray(mesh["eptr"])
    conn = np.asarray(mesh["connectivity"])
    rig = np.where(mid[pid] == 0)[0]
    if len(rig) == 0:
        return np.zeros(0, np.int64)
    idx = np.concatenate([np.arange(eptr[e], eptr[e + 1]) for e in rig])
    return np.unique(conn[idx])


def pulse_records(seed=0, peak_ang=6.0e3, peak_lin=400.0, duration=0.01, t_end=0.03,
                  rate=1.0e4):
    """Seeded synthetic acceleration records in the form of the brain
    drivers' sensor input (six channels of (time s, value)): a half-sine
    angular acceleration of peak ``peak_ang`` rad/s^2 about a random axis plus
    a smaller off-axis half-sine of shifted timing, and a half-sine linear
    acceleration of peak ``peak_lin`` m/s^2 along a random direction, sampled
    at ``rate`` Hz up to ``t_end``."""
    rng = np.random.default_rng(seed)
    t = np.arange(0.0, t_end + 0.5 / rate, 1.0 / rate)

    def half_sine(t0, T):
        x = (t - t0) / T
        return np.where((x >= 0) & (x <= 1), np.sin(np.pi * np.clip(x, 0, 1)), 0.0)

    ax = rng.normal(size=3)
    ax /= np.linalg.norm(ax)
    ax2 = rng.normal(size=3)
    ax2 -= ax2 @ ax * ax
    ax2 /= np.linalg.norm(ax2)
    dl = rng.normal(size=3)
    dl /= np.linalg.norm(dl)
    ang = (peak_ang * np.outer(half_sine(0.0, duration), ax) +
           0.3 * peak_ang * np.outer(half_sine(0.3 * duration, 0.8 * duration), ax2))
    lin = peak_lin * np.outer(half_sine(0.0, 0.8 * duration), dl)
    return [(t.copy(), ang[:, k].copy()) for k in range(3)] + \
           [(t.copy(), lin[:, k].copy()) for k in range(3)]


def head_impact_case(target_elements=2_000_000, seed=0, shell=0.005, **kw):
    """head_case with the outer shell rigid (material 0) as the brain drivers
    model the skull: the shell's nodes follow the rigid-body motion of the
    acceleration records (pulse_records); returns mesh, materials, loads and
    the six records."""
    mesh, mats, _ = head_case(target_elements=target_elements, seed=seed, shell=shell, **kw)
    mid = np.asarray(mats["materialID"]).copy()
    mid[0] = 0  # part 0 is the shell
    mats = dict(materialID=mid.astype(np.int32), properties=mats["properties"])
    loads = Loads(len(mesh["coordinates"]))
    loads.rigid(rigid_nodes(mesh, mats))
    return mesh, mats, loads, pulse_records(seed=seed + 3)


def ensemble_case(n_instances=256, e_min=4_000, e_max=250_000, seed=0, h=1.0e-3, jitter=0.1):
    """Batched ensemble of independent C3D8 Ogden blocks: element counts
    log-uniform in [e_min, e_max], seeded aspect ratios, per-instance
    mu ~ U[0.5, 5] kPa, alpha ~ U[-5, 8] (|alpha| >= 0.1), K ~ U[2, 50] MPa,
    top-face shear amplitude ~ U[0.5, 3] mm at 50 Hz, base fixed.  Returns
    the concatenated mesh, materials (one part per instance), loads and the
    instance node offsets."""
    rng = np.random.default_rng(seed)
    Xs, conns, pids, dofs, fns, parts = [], [], [], [], [], []
    node_off = [0]
    for i in range(n_instances):
        E = int(np.exp(rng.uniform(np.log(e_min), np.log(e_max))))
        r = np.exp(rng.uniform(np.log(0.5), np.log(2.0), 2))  # aspect ratios x:z, y:z
        nz = max(2, int(round((E / (r[0] * r[1])) ** (1.0 / 3.0))))
        nx, ny = max(2, int(round(r[0] * nz))), max(2, int(round(r[1] * nz)))
        mu = rng.uniform(0.5e3, 5.0e3)
        alpha = rng.uniform(-5.0, 8.0)
        while abs(alpha) < 0.1:
            alpha = rng.uniform(-5.0, 8.0)
        K = rng.uniform(2.0e6, 50.0e6)
        amp = rng.uniform(0.5e-3, 3.0e-3)
        m, mt, ld = ogden_block_case(nx=nx, ny=ny, nz=nz, lx=nx * h, ly=ny * h, lz=nz * h,
                                     jitter=jitter, seed=seed * 1000 + i, mu=mu, alpha=alpha,
                                     K=K, amp=amp)
        Xs.append(m["coordinates"])
        conns.append(m["connectivity"] + node_off[-1])
        pids.append(np.full(len(m["etype"]), i, np.int32))
        parts.append((6, list(mt["properties"][:4])))
        d = ld.dof_fn.copy()
        d[d >= 0] += len(fns)
        dofs.append(d)
        fns += ld.fns
        node_off.append(node_off[-1] + len(m["coordinates"]))
    E = sum(len(c) // 8 for c in conns)
    mesh = dict(coordinates=np.concatenate(Xs), connectivity=np.concatenate(conns).astype(np.int32),
                eptr=np.arange(0, 8 * E + 1, 8, dtype=np.int64).astype(np.int32),
                etype=np.zeros(E, np.int32), pid=np.concatenate(pids))
    loads = Loads(node_off[-1])
    loads.dof_fn = np.concatenate(dofs)
    loads.fns = fns
    return mesh, materials(parts), loads, np.array(node_off, np.int32)


def ogden_block_case(nx=200, ny=200, nz=100, lx=0.2, ly=0.2, lz=0.1, jitter=0.1, seed=0,
                     mu=1.5e3, alpha=5.0, K=20e6, rho=1040.0, amp=1e-3, freq=50.0):
    """Jittered C3D8 block under top-face sinusoidal shear, 1-term Ogden
    (the 200x200x100, 4.0M-element scale configuration by default)."""
    mesh = hex_block(nx, ny, nz, lx, ly, lz, jitter=jitter, seed=seed)
    lam = K - 2.0 * mu / 3.0
    mats = materials([(6, [rho, mu, lam, alpha])])
    X = mesh["coordinates"]
    tol = 1e-9
    loads = Loads(len(X))
    loads.fix(np.where(np.abs(X[:, 2]) < tol)[0])
    top = np.where(np.abs(X[:, 2] - lz) < tol)[0]
    loads.sine(top, 0, amp, 2.0 * np.pi * freq)
    loads.fix(top, dofs=(1, 2))
    return mesh, mats, loads
