"""Mesh files: the engine's Abaqus / LS-DYNA reader (native, host only) and
writers of the same formats.

``read_mesh(path)`` returns the arrays a single-rank FemTech run holds after
ReadInputFile + PartitionMesh (src/io/input/ReadInputFile.cpp:26-77,
ReadAbaqus.cpp:26-246, ReadLsDyna.cpp:48-319, PartitionMesh.cpp:485-535) as
the dict the engine and ``meshgen`` use.  The writers produce files those
readers (the reference's and the engine's) read back into the same arrays."""
import ctypes as C

import numpy as np

from . import FtgpuError, lib

_TYPE_NAME = {0: "C3D8", 1: "C3D4", 2: "T3D2"}


class _Mesh(C.Structure):
    _fields_ = [("nNodes", C.c_int), ("nelements", C.c_int), ("ndim", C.c_int),
                ("nPID", C.c_int), ("nPIDglobal", C.c_int), ("missing_nodes", C.c_longlong),
                ("coordinates", C.POINTER(C.c_double)), ("eptr", C.POINTER(C.c_int)),
                ("connectivity", C.POINTER(C.c_int)), ("etype", C.POINTER(C.c_int)),
                ("pid", C.POINTER(C.c_int)), ("global_eid", C.POINTER(C.c_int)),
                ("global_node_id", C.POINTER(C.c_int))]


def read_mesh(path):
    """Read an Abaqus .inp or LS-DYNA .k file: dict(coordinates (nNodes, ndim),
    eptr, connectivity, etype, pid, global_eid, global_node_id, nPID,
    nPIDglobal, missing_nodes)."""
    L = lib()
    L.ftgpu_read_mesh.argtypes = [C.c_char_p, C.POINTER(C.POINTER(_Mesh))]
    L.ftgpu_free_mesh.argtypes = [C.POINTER(_Mesh)]
    L.ftgpu_read_mesh_error.restype = C.c_char_p
    p = C.POINTER(_Mesh)()
    rc = L.ftgpu_read_mesh(str(path).encode(), C.byref(p))
    if rc != 0:
        raise FtgpuError(rc, L.ftgpu_read_mesh_error().decode())
    m = p.contents
    try:
        nN, nE, nd = m.nNodes, m.nelements, m.ndim
        eptr = np.ctypeslib.as_array(m.eptr, (nE + 1,)).copy()
        out = dict(coordinates=np.ctypeslib.as_array(m.coordinates, (max(nN * nd, 1),))[
                       : nN * nd].reshape(nN, nd).copy(),
                   eptr=eptr.astype(np.int32),
                   connectivity=np.ctypeslib.as_array(m.connectivity, (max(int(eptr[-1]), 1),))[
                       : int(eptr[-1])].astype(np.int32).copy(),
                   etype=np.ctypeslib.as_array(m.etype, (nE,)).astype(np.int32).copy(),
                   pid=np.ctypeslib.as_array(m.pid, (nE,)).astype(np.int32).copy(),
                   global_eid=np.ctypeslib.as_array(m.global_eid, (nE,)).astype(np.int32).copy(),
                   global_node_id=np.ctypeslib.as_array(m.global_node_id, (max(nN, 1),))[
                       :nN].astype(np.int32).copy(),
                   nPID=m.nPID, nPIDglobal=m.nPIDglobal, missing_nodes=int(m.missing_nodes))
    finally:
        L.ftgpu_free_mesh(p)
    return out


def _ids(mesh):
    nN = len(mesh["coordinates"])
    nE = len(mesh["eptr"]) - 1
    nid = np.asarray(mesh.get("global_node_id", np.arange(1, nN + 1)))
    eid = np.asarray(mesh.get("global_eid", np.arange(1, nE + 1)))
    return nid, eid


def write_inp(path, mesh, elset_names=None):
    """Abaqus input: one *NODE section, then one *ELEMENT section per run of
    elements with the same type and part (ELSET = the part's name; parts keep
    their numbers when the runs appear in part order)."""
    X = np.asarray(mesh["coordinates"], np.float64)
    eptr, conn = np.asarray(mesh["eptr"]), np.asarray(mesh["connectivity"])
    et, pid = np.asarray(mesh["etype"]), np.asarray(mesh["pid"])
    nid, eid = _ids(mesh)
    names = elset_names or {}
    out = ["*HEADING", "written by femtech_gb300.meshio", "*NODE"]
    out += ["%d, %.17g, %.17g, %.17g" % (nid[i], *X[i]) for i in range(len(X))]
    e = 0
    while e < len(et):
        f = e
        while f < len(et) and et[f] == et[e] and pid[f] == pid[e]:
            f += 1
        out.append("*ELEMENT, TYPE=%s, ELSET=%s" % (_TYPE_NAME[int(et[e])],
                                                     names.get(int(pid[e]), "PART_%d" % pid[e])))
        for k in range(e, f):
            nodes = nid[conn[eptr[k]:eptr[k + 1]]]
            out.append("%d, " % eid[k] + ", ".join(str(int(n)) for n in nodes))
        e = f
    out.append("*END STEP")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


def write_k(path, mesh):
    """LS-DYNA keyword input: *NODE with the column comment the reader keys on,
    *ELEMENT_SOLID with 8 node columns (a C3D4 repeats its last node, which
    the reader drops), part = pid + 1."""
    X = np.asarray(mesh["coordinates"], np.float64)
    eptr, conn = np.asarray(mesh["eptr"]), np.asarray(mesh["connectivity"])
    pid = np.asarray(mesh["pid"])
    nid, eid = _ids(mesh)
    out = ["*KEYWORD", "*NODE",
           "$#   nid               x               y               z      tc      rc"]
    out += ["%8d %.17g %.17g %.17g 0 0" % (nid[i], *X[i]) for i in range(len(X))]
    out += ["*ELEMENT_SOLID", "$#   eid     pid      n1      n2      n3      n4      n5      n6"
            "      n7      n8"]
    for k in range(len(pid)):
        nodes = [int(n) for n in nid[conn[eptr[k]:eptr[k + 1]]]]
        nodes += [nodes[-1]] * (8 - len(nodes))
        out.append("%8d %7d " % (eid[k], pid[k] + 1) + " ".join("%7d" % n for n in nodes))
    out.append("*END")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


def _cell_args(cell_data, nE):
    names = list(cell_data or {})
    arrs = [np.ascontiguousarray(cell_data[k], np.int32) for k in names]
    if any(len(x) != nE for x in arrs):
        raise ValueError("cell data needs one value per element")
    ptrs = (C.c_void_p * max(1, len(arrs)))(*[x.ctypes.data for x in arrs])
    cnames = (C.c_char_p * max(1, len(names)))(*[k.encode() for k in names])
    return len(names), ptrs, cnames, arrs


def write_vtu_arrays(dir, name, step, mesh, u, a, boundary, Eavg, cell_data=None):
    """The reference's WriteVTU output (results/vtu/<name>.vtu.<step>.0000 and
    results/<name>.<step>.pvtu under dir) from host arrays: u, a per DOF,
    boundary 0/1 per DOF, Eavg 9 per element, cell_data name -> int array."""
    L = lib()
    L.ftgpu_write_vtu_arrays.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int] + \
        [C.c_void_p] * 9 + [C.c_int, C.c_void_p, C.c_void_p]
    X = np.ascontiguousarray(mesh["coordinates"], np.float64).ravel()
    ep = np.ascontiguousarray(mesh["eptr"], np.int32)
    cn = np.ascontiguousarray(mesh["connectivity"], np.int32)
    et = np.ascontiguousarray(mesh["etype"], np.int32)
    pid = np.ascontiguousarray(mesh["pid"], np.int32)
    u = np.ascontiguousarray(u, np.float64).ravel()
    a = np.ascontiguousarray(a, np.float64).ravel()
    b = np.ascontiguousarray(boundary, np.int32).ravel()
    E = np.ascontiguousarray(Eavg, np.float64).ravel()
    nc, ptrs, cnames, keep = _cell_args(cell_data, len(et))
    rc = L.ftgpu_write_vtu_arrays(str(dir).encode(), name.encode(), int(step), len(X) // 3,
                                  len(et), *[x.ctypes.data for x in (X, ep, cn, et, pid, u, a, b, E)],
                                  nc, C.cast(ptrs, C.c_void_p), C.cast(cnames, C.c_void_p))
    if rc != 0:
        raise FtgpuError(rc, "write_vtu_arrays failed")


def write_pvd(dir, name, step, step_times):
    """<dir>/<name without extension>.pvd listing results/<name>.<j>.pvtu for
    j = 0..step with their times (WritePVD)."""
    L = lib()
    L.ftgpu_write_pvd.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_void_p]
    t = np.ascontiguousarray(step_times, np.float64)
    if len(t) < step + 1:
        raise ValueError("step + 1 times needed")
    rc = L.ftgpu_write_pvd(str(dir).encode(), name.encode(), int(step), t.ctypes.data)
    if rc != 0:
        raise FtgpuError(rc, "write_pvd failed")
