"""Gmsh MSH 2.x reader (host, no GPU)."""
import numpy as np
import pytest

from probabilistic_peridynamics_gb300.mesh import (MeshFormatError, read_mesh,
                                                   read_msh)

MSH = """$MeshFormat
2.2 0 8
$EndMeshFormat
$PhysicalNames
1
2 1 "plate"
$EndPhysicalNames
$Nodes
5
10 0 0 0
20 1 0 0
30 1 1 0
40 0 1 0
50 0.5 0.5 0.25
$EndNodes
$Elements
6
1 15 2 0 1 10
2 1 2 0 1 10 20
3 2 2 1 5 10 20 50
4 2 2 1 5 20 30 50
5 1 2 0 2 20 30
6 4 2 0 7 10 20 30 50
$EndElements
"""


def test_reads_nodes_and_groups_elements(tmp_path):
    p = tmp_path / "m.msh"
    p.write_text(MSH)
    mesh = read_msh(p)
    assert mesh.points.shape == (5, 3)
    assert np.array_equal(mesh.points[4], [0.5, 0.5, 0.25])
    # node ids 10..50 map to positions 0..4, elements grouped in file order
    assert np.array_equal(mesh.cells_dict["triangle"], [[0, 1, 4], [1, 2, 4]])
    assert np.array_equal(mesh.cells_dict["line"], [[0, 1], [1, 2]])
    assert np.array_equal(mesh.cells_dict["vertex"], [[0]])
    assert np.array_equal(mesh.cells_dict["tetra"], [[0, 1, 2, 4]])
    assert np.array_equal(read_mesh(p).points, mesh.points)


def test_rejects_unsupported_files(tmp_path):
    p = tmp_path / "b.msh"
    p.write_text(MSH.replace("2.2 0 8", "2.2 1 8"))
    with pytest.raises(MeshFormatError):
        read_msh(p)
    p.write_text(MSH.replace("2.2 0 8", "4.1 0 8"))
    with pytest.raises(MeshFormatError):
        read_msh(p)
    p.write_text(MSH.replace("3 2 2 1 5 10 20 50", "3 2 2 1 5 10 20 60"))
    with pytest.raises((MeshFormatError, IndexError)):
        read_msh(p)


# ------------------------------------------------- the reference's meshes
def _reference_data():
    """The reference checkout's test data and example meshes, where the
    checkout is present (read-only; the build container)."""
    from oracle.build_ref import DEFAULT_REFERENCE
    root = DEFAULT_REFERENCE
    if not (root / "peripy" / "test" / "data").is_dir():
        pytest.skip("the reference checkout is not present")
    return root


def _count_msh(path):
    """Node count and element counts by Gmsh type code, read from the file
    with a separate minimal scan (the header counts and each element
    line's second field), to check the reader against."""
    lines = path.read_text().splitlines()
    i = lines.index("$Nodes")
    nnodes = int(lines[i + 1])
    first = [float(v) for v in lines[i + 2].split()[1:4]]
    j = lines.index("$Elements")
    nel = int(lines[j + 1])
    types = {}
    for line in lines[j + 2:j + 2 + nel]:
        code = int(line.split()[1])
        types[code] = types.get(code, 0) + 1
    return nnodes, first, types


#: Gmsh element type codes and the cell names of the reader.
_GMSH = {15: "vertex", 1: "line", 2: "triangle", 4: "tetra", 3: "quad"}


@pytest.mark.parametrize("name", [
    "peripy/test/data/example_mesh_transfinite.msh",
    "peripy/test/data/example_mesh_large.msh",
    "examples/example2/1650beam13539.msh"])
def test_reads_the_reference_meshes(name):
    """Every node and every element of the reference's own MSH meshes."""
    path = _reference_data() / name
    nnodes, first, types = _count_msh(path)
    mesh = read_msh(path)
    assert mesh.points.shape == (nnodes, 3)
    assert np.array_equal(mesh.points[0], first)
    for code, count in types.items():
        assert mesh.cells_dict[_GMSH[code]].shape[0] == count
    if name.endswith("1650beam13539.msh"):
        assert nnodes == 13539


def test_transfinite_model_as_the_reference_expects():
    """``Model`` on ``example_mesh_transfinite.msh`` with transfinite=1 and
    volume_total=1.0, the fixture of ``peripy/test/test_model.py:93-104``:
    2116 nodes, node 69 at (0, 0.4888888888888889, 0) (test_model.py:195-201)
    and every volume 1/2116 (test_model.py:271-274)."""
    import probabilistic_peridynamics_gb300 as pp
    from tests.test_model_host import HostIntegrator
    path = _reference_data() / "peripy/test/data/example_mesh_transfinite.msh"

    def displacement_boundary(x):
        return [None, None, None]

    model = pp.Model(path, integrator=HostIntegrator(), horizon=0.1,
                     critical_stretch=0.05,
                     bond_stiffness=18.0 * 0.05 / (np.pi * 0.1 ** 4),
                     is_displacement_boundary=displacement_boundary,
                     transfinite=1, volume_total=1.0)
    assert model.coords.shape == (2116, 3) and model.nnodes == 2116
    assert np.allclose(model.coords[69], [0, 0.4888888888888889, 0])
    assert np.allclose(model.volume, np.ones(2116) / 2116.0)


def test_large_mesh_warns_as_the_reference_expects():
    """``example_mesh_large.msh`` through ``Model`` warns that the set-up
    may take a while (``peripy/test/test_model.py:445-453``)."""
    import probabilistic_peridynamics_gb300 as pp
    from tests.test_model_host import HostIntegrator
    path = _reference_data() / "peripy/test/data/example_mesh_large.msh"
    with pytest.warns(UserWarning, match="this may take a while"):
        pp.Model(path, integrator=HostIntegrator(), horizon=0.1,
                 critical_stretch=1.0, bond_stiffness=1.0)
