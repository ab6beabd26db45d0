"""femtech_gb300 -- GB300 (sm_103a) engine for FemTech's explicit-dynamics hot path.

The compute lives in ``libftgpu.so`` (CUDA kernels behind the C ABI of
``include/ftgpu.h``).  This module is a thin ctypes front-end whose methods
carry the names of the reference functions they replace:

    ShapeFunctions()+AssembleLumpedMass()  -> Model.setup(), Model.mass
    GetForce()                              -> Model.GetForce(u, dt)
    StableTimeStep()                        -> Model.StableTimeStep(u)
    the driver's explicit loop (ex9.cpp)    -> Model.init_explicit(), Model.run()

There is no CPU fallback: if the library is missing or no GPU is present the
calls raise.
"""
import ctypes as C
import os

import numpy as np

from . import meshgen  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libftgpu.so")

FP64, MIXED = 0, 1
C3D8, C3D4 = 0, 1
OK = 0
ERR_MATERIAL, ERR_INPUT, ERR_ALLOC, ERR_DT, ERR_INVERTED = -1, -3, -12, -19, -20
ERR_CUDA, ERR_STATE, ERR_NODEVICE = -30, -31, -32


class FtgpuError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("ftgpu status %d: %s" % (status, msg))
        self.status = status


class Injury(C.Structure):
    """ftgpu_injury: the running record of the injury criteria."""
    _fields_ = [(k, C.c_double) for k in ("max_strain", "max_strain_time", "min_strain",
                                           "min_strain_time", "max_shear", "max_shear_time",
                                           "max_psxsr", "max_psxsr_time")] + \
               [(k, C.c_int) for k in ("max_strain_elem", "min_strain_elem", "max_shear_elem",
                                        "max_psxsr_elem")] + \
               [(k, C.c_double) for k in ("mps95", "mps95_time", "mpsxsr95", "mpsxsr95_time")] + \
               [("mps95_count", C.c_int), ("mpsxsr95_count", C.c_int), ("steps", C.c_longlong)]


INJ_MPS15, INJ_MPS30, INJ_PSR120, INJ_PSXSR28, INJ_MPS95, INJ_PSXSR95 = 1, 2, 4, 8, 16, 32


class BcFn(C.Structure):
    _fields_ = [("kind", C.c_int), ("pad", C.c_int), ("p", C.c_double * 8)]


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lib = None


def lib():
    """Load libftgpu.so (built by femtech_gb300.build / __graft_entry__.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libftgpu.so is not built; run femtech_gb300.build.build() first")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    L.ftgpu_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int]
    L.ftgpu_destroy.argtypes = [vp]
    L.ftgpu_status_string.restype = C.c_char_p
    L.ftgpu_status_string.argtypes = [C.c_int]
    L.ftgpu_last_error.restype = C.c_char_p
    L.ftgpu_set_mesh.argtypes = [vp, C.c_int, C.c_int, _dp, _ip, _ip, _ip, _ip]
    L.ftgpu_set_materials.argtypes = [vp, C.c_int, _ip, _dp]
    L.ftgpu_set_fibers.argtypes = [vp, _dp]
    L.ftgpu_set_bc.argtypes = [vp, _ip, C.c_int, vp]
    L.ftgpu_set_instances.argtypes = [vp, C.c_int, _ip, _dp, _dp, _dp]
    L.ftgpu_set_patch_size.argtypes = [vp, C.c_int]
    L.ftgpu_setup.argtypes = [vp]
    L.ftgpu_get_mass.argtypes = [vp, _dp]
    L.ftgpu_get_force.argtypes = [vp, _dp, C.c_double, vp, vp]
    L.ftgpu_stable_time_step.argtypes = [vp, _dp, C.POINTER(C.c_double)]
    L.ftgpu_get_gauss_points.argtypes = [vp, vp, vp, vp]
    L.ftgpu_num_gauss_points.argtypes = [vp]
    L.ftgpu_set_state.argtypes = [vp, vp, vp, vp, C.c_double]
    L.ftgpu_init_explicit.argtypes = [vp, C.c_double, C.c_double, C.c_double]
    L.ftgpu_run.argtypes = [vp, C.c_int, C.POINTER(C.c_int)]
    L.ftgpu_get_state.argtypes = [vp, vp, vp, vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                  C.POINTER(C.c_longlong)]
    L.ftgpu_get_instance_clock.argtypes = [vp, vp, vp, vp, vp]
    L.ftgpu_launches_per_step.argtypes = [vp]
    L.ftgpu_check.argtypes = [vp]
    L.ftgpu_set_energy.argtypes = [vp, C.c_int]
    _lib = L
    return L


def _check(status):
    if status != OK:
        L = lib()
        raise FtgpuError(status, "%s (%s)" % (L.ftgpu_status_string(status).decode(),
                                              L.ftgpu_last_error().decode()))


def _ptr(a):
    return None if a is None else a.ctypes.data


def bc_table(fns):
    arr = (BcFn * max(1, len(fns)))()
    for i, (kind, params) in enumerate(fns):
        arr[i].kind = int(kind)
        for j, v in enumerate(params):
            arr[i].p[j] = float(v)
    return arr


class Model:
    """One engine model (mesh + materials + loads) on one GPU."""

    def __init__(self, mesh, mats, precision=MIXED, device=0, fiber=None, loads=None,
                 patch_size=0, instances=None, setup=True):
        L = lib()
        h = C.c_void_p()
        _check(L.ftgpu_create(C.byref(h), int(device), int(precision)))
        self.h = h
        self.precision = precision
        X = np.ascontiguousarray(mesh["coordinates"], np.float64).ravel()
        self.nNodes = len(X) // 3
        eptr = np.ascontiguousarray(mesh["eptr"], np.int32)
        self.nE = len(eptr) - 1
        _check(L.ftgpu_set_mesh(h, self.nNodes, self.nE, X, eptr,
                                np.ascontiguousarray(mesh["connectivity"], np.int32),
                                np.ascontiguousarray(mesh["etype"], np.int32),
                                np.ascontiguousarray(mesh["pid"], np.int32)))
        mid = np.ascontiguousarray(mats["materialID"], np.int32)
        _check(L.ftgpu_set_materials(h, len(mid), mid,
                                     np.ascontiguousarray(mats["properties"], np.float64).ravel()))
        fib = fiber if fiber is not None else mesh.get("fiber")
        if fib is not None:
            _check(L.ftgpu_set_fibers(h, np.ascontiguousarray(fib, np.float64).ravel()))
        if loads is not None:
            self.set_bc(loads.dof_fn, loads.fns)
        if patch_size:
            _check(L.ftgpu_set_patch_size(h, int(patch_size)))
        if instances is not None:
            off = np.ascontiguousarray(instances["node_offset"], np.int32)
            n = len(off) - 1
            _check(L.ftgpu_set_instances(
                h, n, off, np.ascontiguousarray(instances["tmax"], np.float64),
                np.ascontiguousarray(instances["reduction"], np.float64),
                np.ascontiguousarray(instances.get("failure_dt", np.zeros(n)), np.float64)))
        self.ninst = 1 if instances is None else len(instances["node_offset"]) - 1
        if setup:
            self.setup()

    def close(self):
        if getattr(self, "h", None):
            lib().ftgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- set-up ----
    def set_bc(self, dof_fn, fns):
        self._fns = bc_table(fns)
        _check(lib().ftgpu_set_bc(self.h, np.ascontiguousarray(dof_fn, np.int32).ravel(),
                                  len(fns), C.cast(self._fns, C.c_void_p)))

    def setup(self):
        """ShapeFunctions() + AssembleLumpedMass() on the device."""
        _check(lib().ftgpu_setup(self.h))

    @property
    def mass(self):
        m = np.zeros(3 * self.nNodes)
        _check(lib().ftgpu_get_mass(self.h, m))
        return m

    # ---- symbol-compatible primitives ----
    def GetForce(self, u, dt=0.0):
        """Internal force fi (and f_net = -fi) on displacements u, like GetForce()."""
        fi = np.zeros(3 * self.nNodes)
        _check(lib().ftgpu_get_force(self.h, np.ascontiguousarray(u, np.float64).ravel(),
                                     float(dt), fi.ctypes.data, None))
        return fi

    def StableTimeStep(self, u):
        d = C.c_double()
        _check(lib().ftgpu_stable_time_step(self.h, np.ascontiguousarray(u, np.float64).ravel(),
                                            C.byref(d)))
        return d.value

    def gauss_points(self):
        n = lib().ftgpu_num_gauss_points(self.h)
        F, J, S = np.zeros(9 * n), np.zeros(n), np.zeros(6 * n)
        _check(lib().ftgpu_get_gauss_points(self.h, F.ctypes.data, J.ctypes.data, S.ctypes.data))
        return F.reshape(n, 9), J, S.reshape(n, 6)

    # ---- device-resident explicit loop ----
    def set_state(self, u=None, v=None, a=None, time=0.0):
        arrs = [None if x is None else np.ascontiguousarray(x, np.float64).ravel() for x in (u, v, a)]
        _check(lib().ftgpu_set_state(self.h, *[_ptr(x) for x in arrs], float(time)))

    def init_explicit(self, reduction=0.9, failure_dt=0.0, tmax=1e300):
        _check(lib().ftgpu_init_explicit(self.h, float(reduction), float(failure_dt), float(tmax)))

    def run(self, max_steps):
        s = C.c_int()
        _check(lib().ftgpu_run(self.h, int(max_steps), C.byref(s)))
        return s.value

    def state(self, out=None):
        """u, v, a (AoS [node*3+d]), time, dt, step.  out: optional dict of
        preallocated float64 arrays 'u', 'v', 'a' (pinned host memory gives
        full-bandwidth copies); a missing key is not read back."""
        n = 3 * self.nNodes
        if out is not None:
            u, v, a = out.get("u"), out.get("v"), out.get("a")
            t, dt, st = C.c_double(), C.c_double(), C.c_longlong()
            _check(lib().ftgpu_get_state(self.h, _ptr(u), _ptr(v), _ptr(a), C.byref(t),
                                         C.byref(dt), C.byref(st)))
            return dict(u=u, v=v, a=a, time=t.value, dt=dt.value, step=st.value)
        u, v, a = np.zeros(n), np.zeros(n), np.zeros(n)
        t, dt, st = C.c_double(), C.c_double(), C.c_longlong()
        _check(lib().ftgpu_get_state(self.h, u.ctypes.data, v.ctypes.data, a.ctypes.data,
                                     C.byref(t), C.byref(dt), C.byref(st)))
        return dict(u=u, v=v, a=a, time=t.value, dt=dt.value, step=st.value)

    def instance_clocks(self):
        n = self.ninst
        t, dt = np.zeros(n), np.zeros(n)
        st, dn = np.zeros(n, np.int64), np.zeros(n, np.int32)
        _check(lib().ftgpu_get_instance_clock(self.h, t.ctypes.data, dt.ctypes.data,
                                              st.ctypes.data, dn.ctypes.data))
        return dict(time=t, dt=dt, step=st, done=dn)

    def set_surrogate(self, surrogate, trust_e2=0.04):
        """Use a trained femtech_gb300.surrogate.Surrogate for material-7 elements
        (None detaches); Gauss points with |E|_F^2 > trust_e2 use the plain law."""
        L = lib()
        L.ftgpu_set_surrogate.argtypes = [C.c_void_p, C.c_void_p, C.c_double]
        self._surrogate = surrogate
        _check(L.ftgpu_set_surrogate(self.h, None if surrogate is None else surrogate.h,
                                     float(trust_e2)))

    def element_strain(self):
        """CalculateMaximumPrincipalStrain of every element on the current state:
        Eavg [nE, 9] (column-major 3x3), max / min principal strain, max shear."""
        L = lib()
        L.ftgpu_element_strain.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        E9, mx, mn, sh = np.zeros(9 * self.nE), np.zeros(self.nE), np.zeros(self.nE), np.zeros(self.nE)
        _check(L.ftgpu_element_strain(self.h, E9, mx, mn, sh))
        return E9.reshape(-1, 9), mx, mn, sh

    def set_injury(self, element_ids):
        """Per-step injury criteria (ex5's CalculateInjuryCriterions) over these
        elements (call before init_explicit; an empty list turns them off)."""
        L = lib()
        L.ftgpu_set_injury.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        ids = np.ascontiguousarray(element_ids, np.int32)
        self._inj_n = len(ids)
        _check(L.ftgpu_set_injury(self.h, len(ids), ids.ctypes.data if len(ids) else None))

    def injury(self):
        """The record (dict), per listed element the flag bits and the last MPS."""
        L = lib()
        L.ftgpu_get_injury.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        rec = Injury()
        n = self._inj_n
        flags, ps = np.zeros(n, np.int32), np.zeros(n)
        _check(L.ftgpu_get_injury(self.h, C.byref(rec), flags.ctypes.data, ps.ctypes.data))
        out = {k: getattr(rec, k) for k, _ in Injury._fields_}
        out["flags"] = flags
        out["ps"] = ps
        return out

    def set_energy(self, enable=True):
        """Track CheckEnergy's balance in the device loop (call before init_explicit)."""
        _check(lib().ftgpu_set_energy(self.h, int(bool(enable))))

    def energy(self):
        """Cumulative internal / external work, kinetic energy, worst balance ratio, violations."""
        L = lib()
        L.ftgpu_get_energy.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 4 + [
            C.POINTER(C.c_longlong)]
        wi, we, ke, mx = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        nv = C.c_longlong()
        _check(L.ftgpu_get_energy(self.h, C.byref(wi), C.byref(we), C.byref(ke), C.byref(mx),
                                  C.byref(nv)))
        return dict(internal_work=wi.value, external_work=we.value, kinetic=ke.value,
                    max_violation=mx.value, violations=nv.value)

    def set_rigid_body(self, channels, centre=None, inst=0):
        """Acceleration records of instance ``inst``'s rigid body: six (times,
        values) pairs, angular x, y, z (rad/s^2) then linear x, y, z (m/s^2);
        ``channels=None`` removes them (call before init_explicit)."""
        L = lib()
        L.ftgpu_set_rigid_body.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
        if channels is None:
            _check(L.ftgpu_set_rigid_body(self.h, int(inst), None, None, None, None))
            return
        tabs = [(np.ascontiguousarray(t, np.float64), np.ascontiguousarray(v, np.float64))
                for t, v in channels]
        if len(tabs) != 6 or any(len(t) != len(v) for t, v in tabs):
            raise ValueError("six (times, values) channels of equal lengths")
        n = (C.c_int * 6)(*[len(t) for t, _ in tabs])
        tp = (C.c_void_p * 6)(*[t.ctypes.data for t, _ in tabs])
        vp = (C.c_void_p * 6)(*[v.ctypes.data for _, v in tabs])
        c = None if centre is None else np.ascontiguousarray(centre, np.float64)
        _check(L.ftgpu_set_rigid_body(self.h, int(inst), n, tp, vp,
                                      None if c is None else c.ctypes.data))

    def rigid_body(self, inst=0):
        """Integrator state (y, yd) of instance ``inst``'s rigid body:
        y = [omega, r, v_cm, x_cm], yd = dy/dt at the current time."""
        L = lib()
        L.ftgpu_get_rigid_body.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
        y, yd = np.zeros(12), np.zeros(12)
        _check(L.ftgpu_get_rigid_body(self.h, int(inst), y, yd))
        return y, yd

    def write_vtu(self, dir, name, step, cell_data=None):
        """The reference's WriteVTU output of the current state (deformed
        points, displacements, accelerations, boundary flags, parts, the
        averaged strain computed on the device, extra int cell arrays)."""
        from .meshio import _cell_args
        L = lib()
        L.ftgpu_write_vtu.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int,
                                      C.c_void_p, C.c_void_p]
        nc, ptrs, cnames, keep = _cell_args(cell_data, self.nE)
        _check(L.ftgpu_write_vtu(self.h, str(dir).encode(), name.encode(), int(step), nc,
                                 C.cast(ptrs, C.c_void_p), C.cast(cnames, C.c_void_p)))

    def launches_per_step(self):
        return lib().ftgpu_launches_per_step(self.h)

    def check(self):
        _check(lib().ftgpu_check(self.h))
