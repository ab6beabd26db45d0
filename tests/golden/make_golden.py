"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in a checkout where the reference tree exists (the oracle Makefile's
default, or FEMTECH_REFERENCE): it builds the reference's own hot-path
sources into oracle/_ref/libfemtech_ref.so (oracle/Makefile) and records their
outputs on small seeded inputs.  The fixtures are committed; tests never need
the reference tree.

Fixtures:
  ref_force.npz   GetForce / mass / StableTimeStep / Gauss-point pk2 of the
                  reference on jittered C3D8 and C3D4 meshes, materials 1-5,
                  including three consecutive viscoelastic calls (material 5);
                  for material 1 also CalculateMaximumPrincipalStrain of every
                  element (Eavg[9], max / min principal strain, max shear);
                  the 95th percentile (math.cpp, both implementations) of five
                  seeded arrays (pct_data_i, pct_ref_i).
  ref_ex9.npz     examples/ex9 (one C3D8, Neo-Hookean, ramped tension, 0.8
                  dt factor, t = 0..1 s) run by the reference loop, plus the
                  last row of examples/ex9/abaqus/abaqus.rpt (the CI target of
                  examples/ex9/compareResults.py).
  ref_cube.npz    the CPU-runnable configuration: 10x10x10 C3D8 cube 0.01 m,
                  Neo-Hookean rho 1000, mu 3.4 kPa, K 2 MPa, z=0 fixed, top
                  face ramped to 10 % strain over 10 ms, 0.9 dt factor, all
                  displacements every 100 steps, and per step the internal
                  work, external work and kinetic energy of the reference's
                  CheckEnergy (the only energy run of the process, so its
                  works start from zero).
  ref_reader.npz  the reference's mesh readers (ReadAbaqus / ReadLsDyna on one
                  rank, then PartitionMesh's single-rank renumbering) on
                  seeded mixed C3D8/C3D4 meshes written as .inp and .k, and on
                  hand-written files with the formats' corner cases (comments,
                  continued keyword lines, inherited element sets, node ID
                  gaps and unused nodes, degenerate hexahedra, zero node slots,
                  trusses, other element types, CRLF endings); the file texts
                  are stored with the arrays.
  ref_vtu.npz     the reference's WriteVTU + WritePVD files (.vtu, .pvtu,
                  .pvd texts) for a mixed C3D8/C3D4 mesh with a seeded state
                  (displacements below 1e-20 included), boundary flags,
                  averaged strains and two extra cell arrays, for an output
                  name without and with an extension.
  ref_rigid.npz   the rigid-body helpers of the brain drivers on the
                  reference's math.cpp: interpolateLinear on tables with
                  duplicate and uneven times (queries below, at, between and
                  above the samples), and the per-node kinematics of
                  ApplyAccBoundaryConditions (ex5.cpp:345-371, restated in the
                  shim over the reference's quaternion helpers) for seeded
                  integrator states, the zero rotation included.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from femtech_gb300 import meshgen as mg  # noqa: E402
from oracle import oracle as orc  # noqa: E402

# the reference checkout (None where absent: the mesh builders below are
# imported by tests that do not need it)
REF = orc.reference_tree()

MATS = {
    1: [1000.0, 3400.0, 2.0e6],
    2: [1000.0, 3400.0, 2.0e6],
    3: [1000.0, 3400.0, 2.0e6],
    4: [1040.0, 1.0e3, 2.0e6, 5.0e3, 10.0],
    5: [1040.0, 1.0e3, 2.0e6, 5.0e3, 10.0, 0.6, 6.0e-3, 0.2, 2.0e-3],
}


def small_meshes():
    hexm = mg.hex_block(3, 2, 2, 0.003, 0.002, 0.002, jitter=0.15, seed=11)
    tetm = mg.tet_ellipsoid(0.004, 0.003, 0.0025, 0.0012, jitter=0.1, seed=5)
    return hexm, tetm


def force_cases():
    out = {}
    hexm, tetm = small_meshes()
    rng = np.random.default_rng(1234)
    for name, mesh in (("hex", hexm), ("tet", tetm)):
        n = len(mesh["coordinates"])
        # three displacement states, small against the thinnest element
        amp = 3.0e-5 if name == "hex" else 2.0e-6
        u = rng.normal(0.0, amp, (3, 3 * n))
        out[name + "_X"] = mesh["coordinates"]
        out[name + "_conn"] = mesh["connectivity"]
        out[name + "_etype"] = mesh["etype"]
        out[name + "_u"] = u
        for mid, props in MATS.items():
            mats = mg.materials([(mid, props)])
            r = orc.RefBuild(mesh, mats)
            fis, pk2s, strains = [], [], []
            for k in range(3):
                fis.append(r.get_force(u[k], 1.0e-6))
                pk2s.append(r.gp_arrays()[2])
                assert np.all(np.isfinite(fis[-1])), (name, mid, k)
                if mid == 1:  # CalculateMaximumPrincipalStrain on this state's F
                    E9, mx, mn, sh = r.element_strain()
                    strains.append(np.concatenate([E9, mx[:, None], mn[:, None], sh[:, None]], 1))
            out["%s_m%d_fi" % (name, mid)] = np.array(fis)
            out["%s_m%d_pk2" % (name, mid)] = np.array(pk2s)
            if strains:
                out["%s_strain" % name] = np.array(strains)
            out["%s_m%d_mass" % (name, mid)] = r.mass
            b = np.zeros(3 * n, np.int32)
            out["%s_m%d_dt" % (name, mid)] = np.array([r.stable_time_step(u[k], b) for k in range(3)])
    return out


def percentile_cases():
    """The reference's 95th percentiles (math.cpp) of seeded arrays: normal,
    rounded (ties), non-negative, tiny."""
    rng = np.random.default_rng(95)
    out = {}
    arrays = [rng.normal(size=1000), np.round(rng.uniform(0.0, 3.0, 777), 1),
              np.abs(rng.normal(size=12345)), rng.normal(size=21), rng.normal(size=20)]
    for i, d in enumerate(arrays):
        a, b = orc.RefBuild.percentile95(d)
        assert a == b
        out["pct_data_%d" % i] = d
        out["pct_ref_%d" % i] = np.array(a)
    return out


READER_INP_QUIRKS = """** corner cases of the Abaqus reader
*Heading
 quirks
*Node, nset=all
      7,   0.,   0.,   0.
      9,   1.,   0.,   0.
     12,   1.,   1.,   0.
     13,   0.,   1.,   0.
     20,   0.,   0.,   1.
     21,   1.,   0.,   1.
     22,   1.,   1.,   1.
     23,   0.,   1.,   1.
     30,   0.5,  0.5,  2.
     31,   9.,   9.,   9.
     40,   2.,   0.,   0.
*Element, type=C3D8,
 elset=BLOCK
 101, 7, 9, 12, 13, 20, 21, 22, 23
*ELEMENT, TYPE=C3D4
 102, 20, 21, 22, 30
 103, 20, 22, 23, 30
*element, type=T3D2, elset=TRUSS
 104, 9, 40
*Element, type=C3D8R, elset=BLOCK
 105, 7, 9, 12, 13, 20, 21, 22, 23
*End Step
"""

READER_K_QUIRKS = """$ corner cases of the LS-DYNA reader
*KEYWORD
*NODE
$#   nid               x               y               z      tc      rc
       5             0.0             0.0             0.0       0       0
       6             1.0             0.0             0.0       0       0
       8             1.0             1.0             0.0       0       0
       9             0.0             1.0             0.0       0       0
      11             0.0             0.0             1.0       0       0
      12             1.0             0.0             1.0       0       0
      14             1.0             1.0             1.0       0       0
      15             0.0             1.0             1.0       0       0
      17             0.5             0.5             2.0       0       0
      18             3.0             3.0             3.0       0       0
*ELEMENT_SOLID
$#   eid     pid      n1      n2      n3      n4      n5      n6      n7      n8
      41       2       5       6       8       9      11      12      14      15
      42       1      11      12      14      17      17      17      17      17
      43       1      11      14      15      17       0       0       0       0
*ELEMENT_SOLID
$#   eid     pid      n1      n2      n3      n4      n5      n6      n7      n8
      44       3      11      12      14      14      17      17      17      17
*ELEMENT_BEAM
$#   eid     pid      n1      n2
      45       4       6      18
*END
"""


def reader_cases():
    """The reference's readers on written meshes and corner-case files."""
    import tempfile
    from femtech_gb300 import meshio
    out = {}
    rng = np.random.default_rng(7)
    hexm = mg.hex_block(3, 2, 2, 0.03, 0.02, 0.02, jitter=0.1, seed=3)
    tetm = mg.tet_ellipsoid(0.02, 0.015, 0.01, 0.006, jitter=0.1, seed=4)
    nh = len(hexm["coordinates"])
    mix = dict(coordinates=np.vstack([hexm["coordinates"], tetm["coordinates"] + [0.05, 0, 0]]),
               eptr=np.concatenate([hexm["eptr"][:-1], hexm["eptr"][-1] + tetm["eptr"]]),
               connectivity=np.concatenate([hexm["connectivity"], tetm["connectivity"] + nh]),
               etype=np.concatenate([hexm["etype"], tetm["etype"]]),
               pid=np.concatenate([np.zeros(len(hexm["etype"]), np.int32),
                                   1 + (rng.random(len(tetm["etype"])) < 0.5).astype(np.int32)]))
    order = np.argsort(mix["pid"], kind="stable")  # element sets in part order
    nE = len(order)
    ep, cn = [0], []
    for e in order:
        cn.extend(mix["connectivity"][mix["eptr"][e]:mix["eptr"][e + 1]])
        ep.append(len(cn))
    mix.update(eptr=np.array(ep, np.int32), connectivity=np.array(cn, np.int32),
               etype=mix["etype"][order], pid=mix["pid"][order])
    nN = len(mix["coordinates"])
    mix["global_node_id"] = 10 + 3 * np.arange(nN)          # ID gaps
    mix["global_eid"] = 1000 + 2 * np.arange(nE)
    with tempfile.TemporaryDirectory() as d:
        files = []
        for ext, writer in ((".inp", meshio.write_inp), (".k", meshio.write_k)):
            p = os.path.join(d, "mixed" + ext)
            writer(p, mix)
            files.append(("mixed" + ext, open(p).read()))
        files.append(("quirks.inp", READER_INP_QUIRKS))
        files.append(("quirks_crlf.inp", READER_INP_QUIRKS.replace("\n", "\r\n")))
        files.append(("quirks.k", READER_K_QUIRKS))
        for i, (name, text) in enumerate(files):
            p = os.path.join(d, name)
            with open(p, "w", newline="") as fh:
                fh.write(text)
            r = orc.RefBuild.read_mesh(p)
            out["reader_name_%d" % i] = np.array(name)
            out["reader_text_%d" % i] = np.array(text)
            for k, v in r.items():
                out["reader_%s_%d" % (k, i)] = np.asarray(v)
    return out


def vtu_mesh():
    """The mixed mesh of the VTU fixtures (also rebuilt by the tests)."""
    hexm = mg.hex_block(2, 2, 1, 0.02, 0.02, 0.01, jitter=0.1, seed=5)
    nh = len(hexm["coordinates"])
    X = np.vstack([hexm["coordinates"], [[0.005, 0.005, 0.02], [0.015, 0.01, 0.02]]])
    tets = np.array([[nh - 9, nh - 8, nh - 6, nh], [nh - 8, nh - 5, nh - 6, nh + 1]], np.int32)
    conn = np.concatenate([hexm["connectivity"], tets.ravel()])
    eptr = np.concatenate([hexm["eptr"], hexm["eptr"][-1] + 4 * np.arange(1, 3)]).astype(np.int32)
    return dict(coordinates=X, eptr=eptr, connectivity=conn.astype(np.int32),
                etype=np.array([0] * 4 + [1] * 2, np.int32),
                pid=np.array([0, 0, 1, 1, 2, 2], np.int32))


def vtu_state(mesh):
    rng = np.random.default_rng(263)
    n3, nE = 3 * len(mesh["coordinates"]), len(mesh["etype"])
    u = rng.normal(0, 1e-3, n3)
    u[::7] = rng.normal(0, 1e-22, len(u[::7]))  # below the writer's flush threshold
    a = rng.normal(0, 10.0, n3)
    b = (rng.random(n3) < 0.3).astype(np.int32)
    E = rng.normal(0, 0.05, 9 * nE)
    cells = {"MPS-95": (rng.random(nE) < 0.5).astype(np.int32),
             "CSDM-15": rng.integers(0, 2, nE).astype(np.int32)}
    return u, a, b, E, cells


def vtu_cases():
    import tempfile
    mesh = vtu_mesh()
    u, a, b, E, cells = vtu_state(mesh)
    mats = mg.materials([(1, [1000.0, 3400.0, 2.0e6])] * 3)
    r = orc.RefBuild(mesh, mats)
    times = np.array([0.0, 1.25e-3, 2.5e-3, 3.75e-3])
    out = {}
    for i, name in enumerate(("head", "head.inp")):
        with tempfile.TemporaryDirectory() as d:
            r.write_vtu(d, name, 3, u, a, b, E, cells, times)
            base = name.rsplit(".", 1)[0]
            for key, rel in (("vtu", "results/vtu/%s.vtu.0003.0000" % name),
                             ("pvtu", "results/%s.0003.pvtu" % name), ("pvd", base + ".pvd")):
                out["vtu_%s_%d" % (key, i)] = np.array(open(os.path.join(d, rel)).read())
        out["vtu_name_%d" % i] = np.array(name)
    out["vtu_times"] = times
    return out


def rigid_cases():
    rng = np.random.default_rng(339)
    out = {}
    tables = [(np.array([0.0, 1e-3, 1e-3, 2.5e-3, 4e-3, 7e-3, 1e-2]),
               np.array([0.0, 3.0, 5.0, -2.0, 4.5, 4.5, 1.0])),
              (np.array([2e-3]), np.array([7.0])),
              (np.array([0.0, 5e-3]), np.array([-1.0, 2.0]))]
    for i, (x, y) in enumerate(tables):
        q = np.concatenate([[x[0] - 1e-3, x[0], x[-1], x[-1] + 1e-3], x,
                            0.5 * (x[1:] + x[:-1]), rng.uniform(x[0], x[-1], 20)])
        out["interp_x_%d" % i] = x
        out["interp_y_%d" % i] = y
        out["interp_q_%d" % i] = q
        out["interp_ref_%d" % i] = np.array([orc.RefBuild.interp_linear(x, y, v) for v in q])
    ys, yds = [], []
    for k in range(24):
        y = rng.normal(size=12) * np.array([50, 50, 50, 0, 0, 0, 2, 2, 2, 0.01, 0.01, 0.01])
        mag = [0.0, 1e-12, 0.3, 1.5][k % 4]
        r = rng.normal(size=3)
        y[3:6] = mag * r / np.linalg.norm(r)
        ys.append(y)
        yds.append(rng.normal(size=12) * 1e3)
    X = rng.uniform(-0.1, 0.1, (10, 3))
    res = [orc.RefBuild.rigid_point(y, yd, X) for y, yd in zip(ys, yds)]
    out.update(rigid_y=np.array(ys), rigid_yd=np.array(yds), rigid_X=X,
               rigid_uva=np.array(res))
    return out


def abaqus_last_row(path):
    rows = []
    with open(path) as f:
        for line in f:
            parts = line.split()
            try:
                vals = [float(p) for p in parts]
            except ValueError:
                continue
            if len(vals) >= 13:
                rows.append(vals)
    return np.array(rows[-1])


def ex9_case():
    # examples/ex9/1-elt-cube.k: one C3D8, element nodes 1 2 4 3 5 6 8 7
    X = np.array([[0, 0, 0], [0.005, 0, 0], [0, 0.005, 0], [0.005, 0.005, 0],
                  [0, 0, 0.005], [0.005, 0, 0.005], [0, 0.005, 0.005], [0.005, 0.005, 0.005]],
                 np.float64)
    conn = np.array([0, 1, 3, 2, 4, 5, 7, 6], np.int32)
    mesh = dict(coordinates=X, eptr=np.array([0, 8], np.int32), connectivity=conn,
                etype=np.array([0], np.int32), pid=np.array([0], np.int32))
    mats = mg.materials([(1, [1040.0, 100.0, 100.0])])  # examples/ex9/materials.dat
    loads = ex9_loads(X)
    r = orc.RefBuild(mesh, mats)
    res = r.explicit_run(loads.dof_fn, loads.fns, tmax=1.0, reduction=0.8, max_steps=100000,
                         out_every=1)
    abq = abaqus_last_row(os.path.join(REF, "examples/ex9/abaqus/abaqus.rpt"))
    return dict(X=X, conn=conn, u_out=res["u_out"], t_out=res["t_out"], steps=res["steps"],
                time=res["time"], u=res["u"], v=res["v"], a=res["a"],
                abaqus_last=abq[[0, 10, 11, 12]])


def ex9_loads(X):
    """ApplyBoundaryConditions of examples/ex9/ex9.cpp:187-248 (dMax 7 mm, tMax 1 s)."""
    tol = 1e-5
    loads = mg.Loads(len(X))
    fx = np.where(np.abs(X[:, 0]) < tol)[0]
    fy = np.where(np.abs(X[:, 1]) < tol)[0]
    fz = np.where(np.abs(X[:, 2]) < tol)[0]
    top = np.where(np.abs(X[:, 1] - 0.005) < tol)[0]
    loads.fix(fx, dofs=(0,))
    loads.fix(fy, dofs=(1,))
    loads.fix(fz, dofs=(2,))
    loads.ramp(top, 1, 0.007 / 1.0)
    return loads


def cube_case():
    mesh, mats, loads = mg.cube_tension_case(n=10)
    r = orc.RefBuild(mesh, mats)
    res = r.explicit_run(loads.dof_fn, loads.fns, tmax=0.01, reduction=0.9, max_steps=100000,
                         out_every=100, energy=True)
    return dict(u_out=res["u_out"], t_out=res["t_out"], steps=res["steps"], time=res["time"],
                u=res["u"], v=res["v"], a=res["a"], energy=res["energy"])


def main():
    if REF is None:
        raise SystemExit("no reference tree: set FEMTECH_REFERENCE to a FemTech checkout")
    orc.build()
    if not orc.RefBuild.available():
        raise SystemExit("reference build missing")
    np.savez_compressed(os.path.join(HERE, "ref_force.npz"), **force_cases(),
                        **percentile_cases())
    np.savez_compressed(os.path.join(HERE, "ref_ex9.npz"), **ex9_case())
    np.savez_compressed(os.path.join(HERE, "ref_cube.npz"), **cube_case())
    np.savez_compressed(os.path.join(HERE, "ref_rigid.npz"), **rigid_cases())
    np.savez_compressed(os.path.join(HERE, "ref_reader.npz"), **reader_cases())
    np.savez_compressed(os.path.join(HERE, "ref_vtu.npz"), **vtu_cases())
    for f in ("ref_force.npz", "ref_ex9.npz", "ref_cube.npz", "ref_rigid.npz", "ref_reader.npz",
              "ref_vtu.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
