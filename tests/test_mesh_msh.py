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
