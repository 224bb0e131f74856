"""PeriPy's CPU ``Euler`` integrator on the GPU (``integrators.Euler``,
``pp_cy_*``).

Bar: bit-identical to the reference's own compiled ``peripy/peridynamics.pyx``
(``oracle/_ref``, pinned to the Cython-layout goldens by
``test_oracle_c.py``) on every output array -- displacements, forces,
damage, the whole neighbour list (stale entries behind the counts
included) and the counts -- on the reference regression plate, on a
lattice where bonds break in tension and in compression with force
boundary conditions, and through ``Model.simulate``.
"""
import numpy as np
import pytest

from tests.conftest import cuda_available
from tests.cython_setup import (breaking_lattice, cython_plate,
                                 run_gpu_euler, run_reference_euler)
from tests.plate_setup import (BOND_STIFFNESS, CRITICAL_STRETCH, DISP_MAGS,
                               DT, STEPS)

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]


@pytest.fixture(scope="module")
def ref():
    from oracle import build_ref
    if not build_ref.build(quiet=True):
        pytest.skip("the compiled reference is not available")
    return build_ref.load()


def _same(got, want):
    for g, w in zip(got, want):
        assert np.array_equal(g, w, equal_nan=True)


@pytest.mark.parametrize("fused", [True, False])
def test_regression_plate(golden, ref, fused):
    """test_integrators.py:150-195 on the GPU: 10 steps of the cracked
    plate in the Cython layout."""
    setup = cython_plate(golden)
    got = run_gpu_euler(setup, STEPS, DISP_MAGS, DT, BOND_STIFFNESS,
                        CRITICAL_STRETCH, fused=fused)
    _same(got, run_reference_euler(ref, setup, STEPS, DISP_MAGS, DT,
                                   BOND_STIFFNESS, CRITICAL_STRETCH))
    assert np.array_equal(got[3], golden["cy_nlist_crack"])
    assert np.array_equal(got[4], golden["cy_n_neigh_crack"])
    assert np.allclose(got[0], golden["euler_u"])
    assert np.allclose(got[1], golden["euler_force"])
    assert np.allclose(got[2], golden["euler_damage"])


@pytest.mark.parametrize("fused", [True, False])
def test_breaking_lattice_with_force_boundaries(ref, fused):
    """Bonds break in tension (pulled faces) and in compression (the
    loaded top face) and are swap-removed from both rows, many per row."""
    setup = breaking_lattice()
    steps = 60
    mags = 2e-3 * np.arange(1, steps + 1)
    fmags = 0.05 * np.arange(1, steps + 1)
    args = (setup, steps, mags, 0.5, 0.05, 0.01)
    got = run_gpu_euler(*args, fmags=fmags, fused=fused)
    want = run_reference_euler(ref, *args, fmags=fmags)
    _same(got, want)
    broken = int(setup["family"].sum() - want[4].sum())
    assert broken > 100
    # the rows were compacted by the swap-remove rule: stale entries remain
    n_neigh = want[4]
    stale = [want[3][i, n_neigh[i]:setup["family"][i]]
             for i in range(len(n_neigh))]
    assert any(len(s) for s in stale)


def test_model_simulate(golden, tmp_path, ref):
    """Model(..., integrator=Euler(dt)).simulate(...) with the reference's
    regression setup: the compact layout, and the same result as the
    compiled reference step on the model's own connectivity."""
    import probabilistic_peridynamics_gb300 as pp
    from probabilistic_peridynamics_gb300.mesh import write_vtk
    from tests.plate_setup import is_crack, is_displacement_boundary
    mesh = tmp_path / "plate.vtk"
    write_vtk(mesh, golden["points"], [("triangle", golden["cells_triangle"]),
                                       ("line", golden["cells_line"])])
    model = pp.Model(mesh, integrator=pp.Euler(dt=DT), horizon=0.1,
                     critical_stretch=CRITICAL_STRETCH,
                     bond_stiffness=BOND_STIFFNESS,
                     initial_crack=pp.initial_crack_helper(is_crack),
                     is_displacement_boundary=is_displacement_boundary)
    nlist0, n_neigh0 = model.initial_connectivity
    assert nlist0.shape[1] == int(model.family.max())  # compact layout
    u, damage, (nlist, n_neigh), force, ud, _ = model.simulate(
        steps=STEPS, displacement_bc_magnitudes=DISP_MAGS)
    setup = dict(coords=model.coords, volume=model.volume,
                 family=model.family, nlist=nlist0, n_neigh=n_neigh0,
                 bc_types=model.bc_types, bc_values=model.bc_values,
                 force_bc_types=model.force_bc_types,
                 force_bc_values=model.force_bc_values)
    want = run_reference_euler(ref, setup, STEPS, DISP_MAGS, DT,
                               BOND_STIFFNESS, CRITICAL_STRETCH)
    _same((u, force, damage, nlist, n_neigh), want)
    assert np.allclose(u, golden["euler_u"])
