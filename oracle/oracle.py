"""ctypes front-end of the FP64 oracle (test infrastructure only).

Two checkers live here:

* ``Oracle``     -- the C restatement in ``femtech_oracle.c`` (``liboracle.so``),
  built on every machine by ``__graft_entry__.build()``;
* ``RefBuild``   -- the reference's own hot-path sources compiled unmodified
  into ``_ref/libfemtech_ref.so`` (only where the reference tree exists).

Only tests/, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` use
this module; the product package never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REFLIB = os.path.join(HERE, "_ref", "libfemtech_ref.so")

BC_FREE, BC_HOLD = -1, -2
BCK_FIXED, BCK_RAMP, BCK_SINE, BCK_ROT, BCK_RIGID = 0, 1, 2, 3, 4

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class BcFn(C.Structure):
    _fields_ = [("kind", C.c_int), ("pad", C.c_int), ("p", C.c_double * 8)]


class _Injury(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("ids", C.c_void_p), ("ps_old", C.c_void_p), ("psxsr", C.c_void_p),
        ("mps15", C.c_void_p), ("mps30", C.c_void_p), ("psr120", C.c_void_p),
        ("psxsr28", C.c_void_p), ("in_mps95", C.c_void_p), ("in_mpsxsr95", C.c_void_p),
        ("max_strain", C.c_double), ("max_strain_time", C.c_double),
        ("min_strain", C.c_double), ("min_strain_time", C.c_double),
        ("max_shear", C.c_double), ("max_shear_time", C.c_double),
        ("max_psxsr", C.c_double), ("max_psxsr_time", C.c_double),
        ("max_strain_elem", C.c_int), ("min_strain_elem", C.c_int),
        ("max_shear_elem", C.c_int), ("max_psxsr_elem", C.c_int),
        ("mps95", C.c_double), ("mps95_time", C.c_double),
        ("mpsxsr95", C.c_double), ("mpsxsr95_time", C.c_double),
        ("mps95_count", C.c_int), ("mpsxsr95_count", C.c_int),
    ]


INJURY_SCALARS = ("max_strain", "max_strain_time", "max_strain_elem", "min_strain",
                  "min_strain_time", "min_strain_elem", "max_shear", "max_shear_time",
                  "max_shear_elem", "max_psxsr", "max_psxsr_time", "max_psxsr_elem", "mps95",
                  "mps95_time", "mpsxsr95", "mpsxsr95_time", "mps95_count", "mpsxsr95_count")
INJURY_ARRAYS = ("ps_old", "psxsr", "mps15", "mps30", "psr120", "psxsr28", "in_mps95",
                 "in_mpsxsr95")


def _injury_struct(ids):
    ids = np.ascontiguousarray(ids, np.int32)
    n = len(ids)
    arrs = {k: np.zeros(n) for k in ("ps_old", "psxsr")}
    arrs.update({k: np.zeros(n, np.int32) for k in INJURY_ARRAYS[2:]})
    st = _Injury()
    st.n = n
    st.ids = ids.ctypes.data
    for k, a in arrs.items():
        setattr(st, k, a.ctypes.data)
    return st, ids, arrs


def _injury_result(st, arrs):
    out = {k: getattr(st, k) for k in INJURY_SCALARS}
    out.update({k: a.copy() for k, a in arrs.items()})
    return out


class _Rigid(C.Structure):
    _fields_ = [("n", C.c_int * 6), ("t", C.c_void_p * 6), ("v", C.c_void_p * 6),
                ("c", C.c_double * 3), ("y", C.c_double * 12), ("yd", C.c_double * 12)]


class RigidBody:
    """Acceleration records of a rigid body for the oracle: channels = six
    (times, values) pairs, angular x, y, z then linear x, y, z."""

    def __init__(self, channels, centre=(0.0, 0.0, 0.0)):
        self.tabs = [(np.ascontiguousarray(t, np.float64), np.ascontiguousarray(v, np.float64))
                     for t, v in channels]
        assert len(self.tabs) == 6
        self.st = _Rigid()
        for k, (t, v) in enumerate(self.tabs):
            assert len(t) == len(v) and len(t) >= 1
            self.st.n[k] = len(t)
            self.st.t[k] = t.ctypes.data
            self.st.v[k] = v.ctypes.data
        for j in range(3):
            self.st.c[j] = float(centre[j])

    @property
    def y(self):
        return np.array(self.st.y[:])

    @property
    def yd(self):
        return np.array(self.st.yd[:])

    def set_state(self, y, yd):
        for i in range(12):
            self.st.y[i] = float(y[i])
            self.st.yd[i] = float(yd[i])

    def step(self, t, h):
        Oracle.lib().or_rigid_step(C.byref(self.st), C.c_double(t), C.c_double(h))

    def point(self, X):
        """(u, v, a) of the points X (n x 3) under the current state."""
        X = np.ascontiguousarray(X, np.float64).reshape(-1, 3)
        out = np.zeros((3, len(X), 3))
        L = Oracle.lib()
        for i in range(len(X)):
            u, v, a = np.zeros(3), np.zeros(3), np.zeros(3)
            L.or_rigid_point(C.byref(self.st), X[i].copy(), u, v, a)
            out[0, i], out[1, i], out[2, i] = u, v, a
        return out


def interp_linear(x, y, value):
    """The oracle's interpolateLinear (math.cpp:99-119)."""
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    return Oracle.lib().or_interp_linear(len(x), x, y, C.c_double(value))


class _Model(C.Structure):
    _fields_ = [
        ("nNodes", C.c_int), ("nelements", C.c_int), ("nPID", C.c_int),
        ("coordinates", C.c_void_p), ("eptr", C.c_void_p), ("connectivity", C.c_void_p),
        ("etype", C.c_void_p), ("pid", C.c_void_p), ("materialID", C.c_void_p),
        ("properties", C.c_void_p), ("fiber", C.c_void_p),
        ("nGP", C.c_void_p), ("nShp", C.c_void_p), ("gpPtr", C.c_void_p),
        ("dsptr", C.c_void_p), ("gptr", C.c_void_p), ("fptr", C.c_void_p),
        ("pk2ptr", C.c_void_p),
        ("shp", C.c_void_p), ("dshp", C.c_void_p), ("detJ", C.c_void_p), ("gw", C.c_void_p),
        ("F", C.c_void_p), ("detF", C.c_void_p), ("pk2", C.c_void_p),
        ("hist", C.c_void_p), ("mass", C.c_void_p), ("fe", C.c_void_p), ("ce", C.c_void_p),
        ("nthreads", C.c_int),
        ("energy", C.c_void_p), ("energy_cap", C.c_int),
        ("injury", C.c_void_p),
        ("rigid", C.c_void_p),
    ]


def reference_tree():
    """The reference checkout the checker is built from ($FEMTECH_REFERENCE,
    else the Makefile's default), or None where it does not exist."""
    ref = os.environ.get("FEMTECH_REFERENCE")
    if not ref:
        out = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True,
                             text=True)
        ref = out.stdout.strip() if out.returncode == 0 else ""
    return ref if ref and os.path.isdir(os.path.join(ref, "src")) else None


def build(quiet=True):
    """Compile liboracle.so (always) and the reference build (if the tree exists)."""
    out = subprocess.run(["make", "-C", HERE, "liboracle.so"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    ref = reference_tree()
    if ref:
        out = subprocess.run(["make", "-C", HERE, "-j8", "ref", "REF=" + ref],
                             capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError("reference build failed:\n" + out.stdout + out.stderr)


def bc_table(fns):
    """fns: list of (kind, params) -> ctypes array of BcFn."""
    arr = (BcFn * max(1, len(fns)))()
    for i, (kind, params) in enumerate(fns):
        arr[i].kind = kind
        for j, v in enumerate(params):
            arr[i].p[j] = float(v)
    return arr


class Oracle:
    """FP64 restatement of ShapeFunctions/AssembleLumpedMass/GetForce/StableTimeStep."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.exists(LIB):
                build()
            L = C.CDLL(LIB)
            M = C.POINTER(_Model)
            L.or_setup.argtypes = [M]
            L.or_free.argtypes = [M]
            L.or_get_force.argtypes = [M, _dp, C.c_double, _dp]
            L.or_stable_time_step.argtypes = [M, _dp, _ip]
            L.or_stable_time_step.restype = C.c_double
            L.or_material_stress.argtypes = [C.c_int, _dp, _dp, C.c_double, C.c_void_p,
                                             C.c_double, _dp, _dp]
            L.or_explicit_run.argtypes = [M, _ip, C.c_void_p, C.c_int, C.c_double, C.c_double,
                                          C.c_double, C.c_double, C.c_int, C.c_int, _dp, _dp,
                                          _dp, _dp, _dp, C.c_int, C.POINTER(C.c_int),
                                          C.POINTER(C.c_int), C.POINTER(C.c_double),
                                          C.POINTER(C.c_double)]
            L.or_element_strain.argtypes = [M, _dp, _dp, _dp, _dp]
            L.or_percentile95.argtypes = [_dp, C.c_int]
            L.or_percentile95.restype = C.c_double
            L.or_set_threads.argtypes = [M, C.c_int]
            L.or_max_threads.restype = C.c_int
            L.or_interp_linear.argtypes = [C.c_int, _dp, _dp, C.c_double]
            L.or_interp_linear.restype = C.c_double
            L.or_rigid_step.argtypes = [C.c_void_p, C.c_double, C.c_double]
            L.or_rigid_point.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
            cls._lib = L
        return cls._lib

    def __init__(self, mesh, mats, threads=1):
        L = self.lib()
        self.mesh = mesh
        self._keep = {
            "coordinates": np.ascontiguousarray(mesh["coordinates"], dtype=np.float64).ravel(),
            "eptr": np.ascontiguousarray(mesh["eptr"], dtype=np.int32),
            "connectivity": np.ascontiguousarray(mesh["connectivity"], dtype=np.int32),
            "etype": np.ascontiguousarray(mesh["etype"], dtype=np.int32),
            "pid": np.ascontiguousarray(mesh["pid"], dtype=np.int32),
            "materialID": np.ascontiguousarray(mats["materialID"], dtype=np.int32),
            "properties": np.ascontiguousarray(mats["properties"], dtype=np.float64).ravel(),
        }
        fib = mesh.get("fiber")
        if fib is not None:
            self._keep["fiber"] = np.ascontiguousarray(fib, dtype=np.float64).ravel()
        m = _Model()
        m.nNodes = len(self._keep["coordinates"]) // 3
        m.nelements = len(self._keep["eptr"]) - 1
        m.nPID = len(self._keep["materialID"])
        for k, v in self._keep.items():
            setattr(m, k, v.ctypes.data)
        m.nthreads = threads
        self.m = m
        self.nNodes, self.nE = m.nNodes, m.nelements
        rc = L.or_setup(C.byref(m))
        if rc != 0:
            raise RuntimeError("or_setup failed %d" % rc)
        ngp = np.ctypeslib.as_array(C.cast(m.gpPtr, C.POINTER(C.c_int)), (m.nelements + 1,))
        self.ngp_total = int(ngp[-1])

    def set_threads(self, n):
        self.lib().or_set_threads(C.byref(self.m), int(n))

    def __del__(self):
        try:
            self.lib().or_free(C.byref(self.m))
        except Exception:
            pass

    def _arr(self, name, n, ctype=C.c_double):
        return np.ctypeslib.as_array(C.cast(getattr(self.m, name), C.POINTER(ctype)), (n,)).copy()

    @property
    def mass(self):
        return self._arr("mass", 3 * self.nNodes)

    def gp_arrays(self):
        n = self.ngp_total
        return (self._arr("F", 9 * n).reshape(n, 9), self._arr("detF", n),
                self._arr("pk2", 6 * n).reshape(n, 6))

    def shape_arrays(self):
        ds = np.ctypeslib.as_array(C.cast(self.m.dsptr, C.POINTER(C.c_int)), (self.nE + 1,))
        return self._arr("dshp", int(ds[-1])), self._arr("detJ", self.ngp_total)

    def get_force(self, u, dt):
        fi = np.zeros(3 * self.nNodes)
        rc = self.lib().or_get_force(C.byref(self.m), np.ascontiguousarray(u, np.float64).ravel(),
                                     float(dt), fi)
        if rc:
            raise RuntimeError("or_get_force failed %d" % rc)
        return fi

    def stable_time_step(self, u, boundary):
        return self.lib().or_stable_time_step(C.byref(self.m),
                                              np.ascontiguousarray(u, np.float64).ravel(),
                                              np.ascontiguousarray(boundary, np.int32).ravel())

    def element_strain(self):
        """CalculateMaximumPrincipalStrain of every element on the F of the last
        get_force: Eavg [nE, 9] (reference layout), max / min principal strain,
        max shear."""
        E9, mx, mn, sh = _strain_outputs(self.nE)
        self.lib().or_element_strain(C.byref(self.m), E9, mx, mn, sh)
        return E9.reshape(-1, 9), mx, mn, sh

    def explicit_run(self, dof_fn, fns, tmax, reduction, max_steps, out_every, t0=0.0,
                     failure_dt=0.0, u=None, v=None, a=None, max_out=None, energy=False,
                     injury_ids=None, rigid=None):
        """The ex9 loop; energy=True adds per step (Wint, Wext, WKE) of
        CheckEnergy (cumulative works, kinetic energy) as result['energy'];
        injury_ids adds the injury criteria of ex5 over those elements as
        result['injury']; rigid (a RigidBody) drives the BCK_RIGID functions
        (its final state is left in it)."""
        n = 3 * self.nNodes
        inj = None
        if injury_ids is not None:
            inj = _injury_struct(injury_ids)
            self.m.injury = C.addressof(inj[0])
        self.m.rigid = None if rigid is None else C.addressof(rigid.st)
        ebuf = np.zeros(3 * max(max_steps, 1)) if energy else None
        self.m.energy = None if ebuf is None else ebuf.ctypes.data
        self.m.energy_cap = max_steps if energy else 0
        u = np.zeros(n) if u is None else np.array(u, np.float64).ravel()
        v = np.zeros(n) if v is None else np.array(v, np.float64).ravel()
        a = np.zeros(n) if a is None else np.array(a, np.float64).ravel()
        if max_out is None:
            max_out = max(1, max_steps // max(out_every, 1) + 1)
        uo = np.zeros(max_out * n)
        to = np.zeros(max_out)
        nout, steps = C.c_int(), C.c_int()
        tt, dd = C.c_double(), C.c_double()
        tab = bc_table(fns)
        rc = self.lib().or_explicit_run(
            C.byref(self.m), np.ascontiguousarray(dof_fn, np.int32).ravel(), C.cast(tab, C.c_void_p),
            len(fns), t0, tmax, reduction, failure_dt, max_steps, out_every, u, v, a, uo, to,
            max_out, C.byref(nout), C.byref(steps), C.byref(tt), C.byref(dd))
        self.m.energy = None
        self.m.energy_cap = 0
        self.m.injury = None
        self.m.rigid = None
        k = nout.value
        res = dict(rc=rc, u=u, v=v, a=a, u_out=uo[: k * n].reshape(k, n), t_out=to[:k],
                   steps=steps.value, time=tt.value, dt=dd.value)
        if energy:
            res["energy"] = ebuf.reshape(-1, 3)[: steps.value].copy()
        if inj is not None:
            res["injury"] = _injury_result(inj[0], inj[2])
        return res


def _strain_outputs(nE):
    return np.zeros(9 * nE), np.zeros(nE), np.zeros(nE), np.zeros(nE)


def percentile95(data):
    """The oracle's 95th percentile (restating math.cpp:160-196)."""
    d = np.ascontiguousarray(data, np.float64)
    return Oracle.lib().or_percentile95(d, len(d))


def material_stress(mat, props, F, J=None, a0=None, dt=0.0, hist=None):
    """Single-point PK2 stress (Voigt 11,22,33,23,13,12) of the oracle's laws."""
    L = Oracle.lib()
    F = np.ascontiguousarray(F, np.float64).reshape(9)
    if J is None:
        J = float(np.linalg.det(F.reshape(3, 3, order="F")))
    h = np.zeros(27) if hist is None else hist
    S = np.zeros(6)
    a0p = None
    if a0 is not None:
        a0 = np.ascontiguousarray(a0, np.float64)
        a0p = a0.ctypes.data
    pr = np.zeros(9)
    pr[: len(props)] = props
    rc = L.or_material_stress(int(mat), pr, F, float(J), a0p, float(dt), h, S)
    if rc:
        raise RuntimeError("unknown material")
    return S


class RefBuild:
    """The reference's own sources (one rank), as a checker for the oracle."""

    _lib = None

    @classmethod
    def available(cls):
        return os.path.exists(REFLIB)

    @classmethod
    def lib(cls):
        if cls._lib is None:
            L = C.CDLL(REFLIB)
            L.ref_setup.argtypes = [C.c_int, C.c_int, _dp, _ip, _ip, _ip, _ip, C.c_int, _ip, _dp,
                                    C.c_void_p]
            L.ref_get_mass.argtypes = [_dp]
            L.ref_num_gp.restype = C.c_int
            L.ref_get_gp.argtypes = [_dp, _dp, _dp]
            L.ref_get_shape.argtypes = [_dp, _dp]
            L.ref_get_force.argtypes = [_dp, C.c_double, _dp, _dp]
            L.ref_stable_time_step.argtypes = [_dp, _ip]
            L.ref_stable_time_step.restype = C.c_double
            L.ref_set_energy_out.argtypes = [C.c_void_p, C.c_int]
            L.ref_element_strain.argtypes = [_dp, _dp, _dp, _dp]
            L.ref_percentile95.argtypes = [_dp, C.c_int, C.POINTER(C.c_double),
                                           C.POINTER(C.c_double)]
            L.ref_write_vtu.argtypes = [C.c_char_p, C.c_char_p, C.c_int, _dp, _dp, _ip, _dp,
                                        C.c_int, C.c_void_p, C.c_void_p, _dp]
            L.ref_read_mesh.argtypes = [C.c_char_p, C.POINTER(C.c_int)]
            L.ref_mesh_arrays.argtypes = [C.c_void_p] * 7
            L.ref_interp_linear.argtypes = [C.c_int, _dp, _dp, C.c_double]
            L.ref_interp_linear.restype = C.c_double
            L.ref_rigid_point.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp]
            L.ref_explicit_run.argtypes = [_ip, C.c_void_p, C.c_int, C.c_double, C.c_double,
                                           C.c_double, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp,
                                           C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                           C.POINTER(C.c_double), C.POINTER(C.c_double)]
            cls._lib = L
        return cls._lib

    def __init__(self, mesh, mats):
        L = self.lib()
        self.X = np.ascontiguousarray(mesh["coordinates"], np.float64).ravel()
        self.nNodes = len(self.X) // 3
        eptr = np.ascontiguousarray(mesh["eptr"], np.int32)
        self.nE = len(eptr) - 1
        fib = mesh.get("fiber")
        self._fib = None if fib is None else np.ascontiguousarray(fib, np.float64).ravel()
        rc = L.ref_setup(self.nNodes, self.nE, self.X, eptr,
                         np.ascontiguousarray(mesh["connectivity"], np.int32),
                         np.ascontiguousarray(mesh["etype"], np.int32),
                         np.ascontiguousarray(mesh["pid"], np.int32), len(mats["materialID"]),
                         np.ascontiguousarray(mats["materialID"], np.int32),
                         np.ascontiguousarray(mats["properties"], np.float64).ravel(),
                         None if self._fib is None else self._fib.ctypes.data)
        if rc:
            raise RuntimeError("ref_setup failed %d" % rc)
        self.ngp = L.ref_num_gp()

    @property
    def mass(self):
        m = np.zeros(3 * self.nNodes)
        self.lib().ref_get_mass(m)
        return m

    def gp_arrays(self):
        n = self.ngp
        F, d, p = np.zeros(9 * n), np.zeros(n), np.zeros(6 * n)
        self.lib().ref_get_gp(F, d, p)
        return F.reshape(n, 9), d, p.reshape(n, 6)

    def get_force(self, u, dt):
        fi, fn = np.zeros(3 * self.nNodes), np.zeros(3 * self.nNodes)
        rc = self.lib().ref_get_force(np.ascontiguousarray(u, np.float64).ravel(), float(dt), fi, fn)
        if rc:
            raise RuntimeError("ref_get_force failed %d" % rc)
        return fi

    def write_vtu(self, dir, name, step, u, a, boundary, Eavg, cell_data, step_times):
        """The reference's WriteVTU + WritePVD for this mesh and the given
        state into dir (cell_data: dict name -> int array per element)."""
        names = list(cell_data)
        arrs = [np.ascontiguousarray(cell_data[k], np.int32) for k in names]
        ptrs = (C.c_void_p * max(1, len(arrs)))(*[x.ctypes.data for x in arrs])
        cnames = (C.c_char_p * max(1, len(names)))(*[k.encode() for k in names])
        rc = self.lib().ref_write_vtu(str(dir).encode(), name.encode(), int(step),
                                      np.ascontiguousarray(u, np.float64).ravel(),
                                      np.ascontiguousarray(a, np.float64).ravel(),
                                      np.ascontiguousarray(boundary, np.int32).ravel(),
                                      np.ascontiguousarray(Eavg, np.float64).ravel(),
                                      len(names), C.cast(ptrs, C.c_void_p),
                                      C.cast(cnames, C.c_void_p),
                                      np.ascontiguousarray(step_times, np.float64))
        if rc:
            raise RuntimeError("ref_write_vtu failed %d" % rc)

    @classmethod
    def read_mesh(cls, path):
        """The reference's ReadInputFile (ReadAbaqus / ReadLsDyna) on one rank
        plus the single-rank renumbering of PartitionMesh: the arrays of
        femtech_gb300.meshio.read_mesh."""
        L = cls.lib()
        sz = (C.c_int * 5)()
        rc = L.ref_read_mesh(str(path).encode(), sz)
        if rc:
            raise RuntimeError("reference reader failed %d" % rc)
        nN, nE, nd, npg, nc = list(sz)
        X = np.zeros(max(nN * nd, 1))
        ep = np.zeros(nE + 1, np.int32)
        conn = np.zeros(max(nc, 1), np.int32)
        et, pid, eid = (np.zeros(max(nE, 1), np.int32) for _ in range(3))
        gid = np.zeros(max(nN, 1), np.int32)
        L.ref_mesh_arrays(X.ctypes.data, ep.ctypes.data, conn.ctypes.data, et.ctypes.data,
                          pid.ctypes.data, eid.ctypes.data, gid.ctypes.data)
        return dict(coordinates=X[: nN * nd].reshape(nN, nd), eptr=ep, connectivity=conn[:nc],
                    etype=et[:nE], pid=pid[:nE], global_eid=eid[:nE], global_node_id=gid[:nN],
                    nPIDglobal=npg)

    @classmethod
    def interp_linear(cls, x, y, value):
        """The reference's interpolateLinear (math.cpp:99-119)."""
        x = np.ascontiguousarray(x, np.float64).copy()
        y = np.ascontiguousarray(y, np.float64).copy()
        return cls.lib().ref_interp_linear(len(x), x, y, float(value))

    @classmethod
    def rigid_point(cls, y, yd, X):
        """(u, v, a) of the points X (n x 3) by ex5's per-node rigid-body
        kinematics on the reference's quaternion helpers."""
        y = np.ascontiguousarray(y, np.float64)
        yd = np.ascontiguousarray(yd, np.float64)
        X = np.ascontiguousarray(X, np.float64).reshape(-1, 3)
        out = np.zeros((3, len(X), 3))
        for i in range(len(X)):
            u, v, a = np.zeros(3), np.zeros(3), np.zeros(3)
            cls.lib().ref_rigid_point(y, yd, X[i].copy(), u, v, a)
            out[0, i], out[1, i], out[2, i] = u, v, a
        return out

    @classmethod
    def percentile95(cls, data):
        """The reference's compute95thPercentileValueBruteForce and
        compute95thPercentileValue (one rank) of the values."""
        d = np.ascontiguousarray(data, np.float64).copy()
        a, b = C.c_double(), C.c_double()
        rc = cls.lib().ref_percentile95(d, len(d), C.byref(a), C.byref(b))
        if rc:
            raise RuntimeError("ref_percentile95 failed %d" % rc)
        return a.value, b.value

    def element_strain(self):
        """The reference's CalculateMaximumPrincipalStrain on every element (F of
        the last get_force)."""
        E9, mx, mn, sh = _strain_outputs(self.nE)
        rc = self.lib().ref_element_strain(E9, mx, mn, sh)
        if rc:
            raise RuntimeError("ref_element_strain failed %d" % rc)
        return E9.reshape(-1, 9), mx, mn, sh

    def stable_time_step(self, u, boundary):
        return self.lib().ref_stable_time_step(np.ascontiguousarray(u, np.float64).ravel(),
                                               np.ascontiguousarray(boundary, np.int32).ravel())

    def explicit_run(self, dof_fn, fns, tmax, reduction, max_steps, out_every, t0=0.0,
                     max_out=None, energy=False):
        """energy=True: per step (Wint, Wext, WKE) as the reference's CheckEnergy
        logs them (works accumulate over the process: one energy run per process)."""
        n = 3 * self.nNodes
        u, v, a = np.zeros(n), np.zeros(n), np.zeros(n)
        ebuf = np.zeros(3 * max(max_steps, 1)) if energy else None
        self.lib().ref_set_energy_out(None if ebuf is None else ebuf.ctypes.data,
                                      max_steps if energy else 0)
        if max_out is None:
            max_out = max(1, max_steps // max(out_every, 1) + 1)
        uo, to = np.zeros(max_out * n), np.zeros(max_out)
        nout, steps = C.c_int(), C.c_int()
        tt, dd = C.c_double(), C.c_double()
        tab = bc_table(fns)
        rc = self.lib().ref_explicit_run(np.ascontiguousarray(dof_fn, np.int32).ravel(),
                                         C.cast(tab, C.c_void_p), len(fns), t0, tmax, reduction,
                                         max_steps, out_every, u, v, a, uo, to, max_out,
                                         C.byref(nout), C.byref(steps), C.byref(tt), C.byref(dd))
        self.lib().ref_set_energy_out(None, 0)
        k = nout.value
        res = dict(rc=rc, u=u, v=v, a=a, u_out=uo[: k * n].reshape(k, n), t_out=to[:k],
                   steps=steps.value, time=tt.value, dt=dd.value)
        if energy:
            res["energy"] = ebuf.reshape(-1, 3)[: steps.value].copy()
        return res
