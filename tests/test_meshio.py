"""Mesh input: the engine's Abaqus / LS-DYNA reader against the reference's
readers (ReadAbaqus / ReadLsDyna on one rank plus PartitionMesh's single-rank
renumbering).

CPU: the reader is host code in libftgpu.so (no device needed): the
reference's outputs on written meshes and corner-case files
(tests/golden/ref_reader.npz), the reference's own example meshes where the
reference tree and its build exist, write/read round trips and errors.
GPU: a model built from a file runs exactly as one built from the arrays."""
import glob
import os

import numpy as np
import pytest

from femtech_gb300 import meshgen as mg

KEYS = ("coordinates", "eptr", "connectivity", "etype", "pid", "global_eid", "global_node_id",
        "nPIDglobal")


def _same(a, b):
    return [k for k in KEYS if not np.array_equal(np.asarray(a[k]), np.asarray(b[k]))]


@pytest.mark.parametrize("i", range(5))
def test_reader_matches_reference_fixture(golden_reader, tmp_path, i):
    from femtech_gb300 import meshio
    g = golden_reader
    name = str(g["reader_name_%d" % i])
    p = tmp_path / name
    with open(p, "w", newline="") as fh:
        fh.write(str(g["reader_text_%d" % i]))
    got = meshio.read_mesh(p)
    ref = {k: g["reader_%s_%d" % (k, i)] for k in KEYS}
    assert _same(got, ref) == [], name


def test_reader_matches_reference_on_its_example_meshes(oracle_lib):
    """Every .inp / .k under the reference's examples, where the reference
    tree and its build are present (not on a machine without them)."""
    from femtech_gb300 import meshio
    ref = oracle_lib.reference_tree()
    if ref is None or not oracle_lib.RefBuild.available():
        pytest.skip("reference tree / build not present")
    files = sorted(glob.glob(os.path.join(ref, "examples", "**", "*.inp"), recursive=True) +
                   glob.glob(os.path.join(ref, "examples", "**", "*.k"), recursive=True))
    assert files
    for f in files:
        assert _same(meshio.read_mesh(f), oracle_lib.RefBuild.read_mesh(f)) == [], f


@pytest.mark.parametrize("ext", [".inp", ".k"])
def test_write_read_round_trip(tmp_path, ext):
    from femtech_gb300 import meshio
    mesh, mats, _ = mg.head_case(target_elements=3_000, seed=1)
    p = tmp_path / ("head" + ext)
    (meshio.write_inp if ext == ".inp" else meshio.write_k)(p, mesh)
    got = meshio.read_mesh(p)
    assert np.array_equal(got["coordinates"], mesh["coordinates"])
    assert np.array_equal(got["eptr"], mesh["eptr"])
    assert np.array_equal(got["connectivity"], mesh["connectivity"])
    assert np.array_equal(got["etype"], mesh["etype"])
    assert np.array_equal(got["pid"], mesh["pid"])
    assert got["missing_nodes"] == 0 and got["nPID"] == 2


def test_reader_reports_missing_nodes_and_errors(tmp_path):
    from femtech_gb300 import meshio, FtgpuError
    p = tmp_path / "m.inp"
    p.write_text("*NODE\n1, 0., 0., 0.\n2, 1., 0., 0.\n3, 0., 1., 0.\n"
                 "*ELEMENT, TYPE=C3D4, ELSET=A\n1, 1, 2, 3, 4\n")
    got = meshio.read_mesh(p)
    assert got["missing_nodes"] == 1 and np.all(got["coordinates"][3] == 0)
    bad = tmp_path / "m.txt"
    bad.write_text("x")
    with pytest.raises(FtgpuError):
        meshio.read_mesh(bad)
    with pytest.raises(FtgpuError):
        meshio.read_mesh(tmp_path / "absent.inp")
    empty = tmp_path / "e.k"
    empty.write_text("*KEYWORD\n*END\n")
    with pytest.raises(FtgpuError):
        meshio.read_mesh(empty)


@pytest.mark.gpu
def test_model_from_file_runs_as_model_from_arrays(tmp_path):
    import femtech_gb300 as ft
    from femtech_gb300 import meshio
    mesh, mats, loads = mg.head_case(target_elements=6_000, seed=2)
    p = tmp_path / "head.inp"
    meshio.write_inp(p, mesh)
    rd = meshio.read_mesh(p)
    rd["fiber"] = mesh["fiber"]
    us = []
    for m_ in (mesh, rd):
        m = ft.Model(m_, mats, precision=ft.FP64, loads=loads)
        m.init_explicit(0.9, 0.0, 1.0)
        assert m.run(60) == 60
        us.append(m.state()["u"])
        m.close()
    assert np.array_equal(us[0], us[1])
