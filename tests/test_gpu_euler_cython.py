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


def test_known_answers_of_the_cython_functions():
    """The reference's own known answers for peridynamics.pyx
    (test_peridynamics.py:7-57): damage, and break_bonds on the 5-node
    case with its expected compacted rows (critical strain 1.0)."""
    import probabilistic_peridynamics_gb300 as pp
    r0 = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0],
                   [2.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    nl = np.array([[1, 2, 4], [0, 3, 0], [0, 0, 0], [1, 0, 0], [0, 0, 0]],
                  dtype=np.intc)
    n_neigh = np.array([3, 2, 1, 1, 1], dtype=np.intc)
    r = np.array([[0.0, 0.0, 0.0], [2.0, 0.0, 0.0], [0.0, 1.0, 0.0],
                  [3.0, 0.0, 0.0], [0.0, 0.0, 2.0]])
    n = 5
    integ = pp.Euler(1.0)
    z = np.zeros((n, 3))
    integ.build(n, 3, 3, r0, np.ones(n), n_neigh.copy(),
                np.ones((n, 3), dtype=np.intc), z, np.zeros((n, 3), np.intc),
                z, None, None, None)
    # every displacement is a boundary value: one step moves r0 to r, and
    # the next step's breaks see r
    integ.create_buffers(nl.copy(), n_neigh.copy(), 1.0, 1.0, None,
                         np.zeros((n, 3)), z, z, z, z, np.zeros(n), None, 1,
                         1)
    integ._bc_values_d.copy_(torch_tensor(r - r0, integ))
    integ(1.0, 0.0)  # u := r - r0; the breaks of this step saw u = 0
    integ(1.0, 0.0)  # breaks at r
    _, _, _, _, _, damage, got_nl, got_nn = integ.write(*[None] * 8)
    assert np.array_equal(got_nl, [[2, 2, 4], [3, 3, 0], [0, 0, 0],
                                   [1, 0, 0], [0, 0, 0]])
    assert np.array_equal(got_nn, [1, 1, 1, 1, 0])
    family = n_neigh.astype(np.float64)
    assert np.array_equal(damage, (family - got_nn) / family)


def torch_tensor(a, integ):
    import torch
    return torch.as_tensor(a, device=integ.device_context.device)


def test_asymmetric_list_is_rejected():
    """The 3-node list of the reference's force test (test_peridynamics.py
    :92-133) is not symmetric (node 2's row holds itself, node 1's holds
    node 2): the GPU Euler refuses it rather than differ."""
    import probabilistic_peridynamics_gb300 as pp
    n = 3
    r0 = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [1.0, 1.0, 0.0]])
    nl = np.array([[1, 0], [0, 2], [2, 0]], dtype=np.intc)
    n_neigh = np.array([1, 2, 1], dtype=np.intc)
    integ = pp.Euler(1.0)
    z = np.zeros((n, 3))
    integ.build(n, 3, 2, r0, np.full(n, 0.16666667), n_neigh.copy(),
                np.zeros((n, 3), np.intc), z, np.zeros((n, 3), np.intc), z,
                None, None, None)
    with pytest.raises(ValueError, match="symmetric"):
        integ.create_buffers(nl, n_neigh, 1.0, 1.0, None, z, z, z, z, z,
                             np.zeros(n), None, 1, 1)
    # the same bonds listed from both ends are accepted
    sym = np.array([[1, 0], [0, 2], [1, 0]], dtype=np.intc)
    integ.create_buffers(sym, n_neigh, 1.0, 1.0, None, z, z, z, z, z,
                         np.zeros(n), None, 1, 1)
