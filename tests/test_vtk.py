"""Legacy-VTK IO (the pyvista replacement for the mesh input and the output frames): write/read
round trips in both encodings, cell data, and TetraCell loading a written mesh. CPU only."""

import numpy as np
import pytest

from nofluidx3d_gb300.mesh import kuhn_sphere
from nofluidx3d_gb300.vtk import VTK_TETRA, read_vtk, write_vtk


@pytest.mark.parametrize("binary", [False, True])
def test_round_trip(tmp_path, binary):
    m = kuhn_sphere(3.0, 0.02, 4)
    vm = np.linspace(0.0, 1.0, m.num_tetra)
    p = tmp_path / "cell.vtk"
    write_vtk(str(p), m.points, m.tets, {"vonMises": vm, "pressure": -vm}, binary=binary)
    r = read_vtk(str(p))
    np.testing.assert_array_equal(r.points, m.points)
    np.testing.assert_array_equal(r.cells_dict[VTK_TETRA], m.tets)
    assert r.n_cells == m.num_tetra and r.n_points == m.num_points
    np.testing.assert_allclose(r.cell_data["vonMises"], vm, rtol=0, atol=1e-6 if not binary else 0)
    np.testing.assert_allclose(r.cell_data["pressure"], -vm, rtol=0, atol=1e-6 if not binary else 0)


def test_tetracell_reads_a_written_mesh(tmp_path):
    from nofluidx3d_gb300.TetraCell import TetraCell

    m = kuhn_sphere(4.0, 0.02, 1)
    p = tmp_path / "init.vtk"
    write_vtk(str(p), m.points, m.tets)
    cell = TetraCell(str(p), 8.0, True)
    # recentred on point 0 and scaled so that point 1 sits at the new radius (TetraCell.py:16-20)
    np.testing.assert_allclose(cell.points[0], 0.0, atol=1e-12)
    assert np.linalg.norm(cell.points[1]) == pytest.approx(8.0)
    assert cell.tetras.shape == (m.num_tetra, 4)
    assert np.all(cell.volumes > 0)
