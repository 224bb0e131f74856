"""Initial crack on the GPU (``pp_create_crack``).

Bar: bit-identical neighbour list and counts to the sequential loop of
``peripy/create_crack.pyx:1-43``: the reference's own compiled module where
it is built, else the host restatement (which the host tests pin to it).
Cases: the 2113-node plate's crack against the reference's connectivity
golden, seeded adversarial crack lists, the 200x200x10 lattice's plane crack
(30,940 pairs), a bad index part-way through the list, an empty list, and
``Model`` with an ``initial_crack`` on a CUDA integrator.
"""
import numpy as np
import pytest

from tests.conftest import cuda_available
from tests.crack_cases import crack_cases, lattice_rows

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]


def _sequential():
    from oracle import build_ref
    if not build_ref.available():
        build_ref.build(quiet=True)
    if build_ref.available():
        return build_ref.load("create_crack").create_crack
    from probabilistic_peridynamics_gb300.model import create_crack
    return create_crack


def _gpu(crack, nlist, n_neigh):
    from probabilistic_peridynamics_gb300.neighbours import create_crack
    create_crack(crack, nlist, n_neigh)


def test_plate_crack_matches_golden(golden):
    from tests.plate_setup import crack_pairs
    nlist = golden["nlist_basic"].astype(np.intc).copy()
    n_neigh = golden["n_neigh_basic"].astype(np.intc).copy()
    crack = np.array(crack_pairs(golden["points"], nlist, n_neigh),
                     dtype=np.intc)
    _gpu(crack, nlist, n_neigh)
    assert np.array_equal(nlist, golden["euler_nlist"])
    assert np.array_equal(n_neigh, golden["euler_n_neigh"])


@pytest.mark.parametrize("case", range(6))
def test_adversarial_lists_match_sequential(case):
    crack, nlist, n_neigh = crack_cases(case)
    want_nl, want_nn = nlist.copy(), n_neigh.copy()
    _sequential()(crack, want_nl, want_nn)
    _gpu(crack, nlist, n_neigh)
    assert np.array_equal(nlist, want_nl)
    assert np.array_equal(n_neigh, want_nn)


def test_full_size_plane_crack_matches_sequential():
    from probabilistic_peridynamics_gb300 import lattice
    coords = lattice.lattice_coords(200, 200, 10, 0.005)
    nlist, n_neigh = lattice_rows(200, 200, 10, 3.015)
    pairs = lattice.plane_crack_pairs(coords, nlist, n_neigh, 0.5, 0.25)
    assert len(pairs) == 30_940
    crack = np.ascontiguousarray(pairs, dtype=np.intc)
    want_nl, want_nn = nlist.copy(), n_neigh.copy()
    _sequential()(crack, want_nl, want_nn)
    _gpu(crack, nlist, n_neigh)
    assert np.array_equal(n_neigh, want_nn)
    assert np.array_equal(nlist, want_nl)
    assert int(n_neigh.sum()) == 42_700_528 - 2 * 30_940


def test_bad_index_applies_the_pairs_before_it():
    crack, nlist, n_neigh = crack_cases(1)
    bad = crack.copy()
    bad[len(bad) // 2] = (0, nlist.shape[0] + 3)
    want_nl, want_nn = nlist.copy(), n_neigh.copy()
    _sequential()(np.ascontiguousarray(crack[:len(bad) // 2]), want_nl,
                  want_nn)
    with pytest.raises(IndexError):
        _gpu(bad, nlist, n_neigh)
    assert np.array_equal(nlist, want_nl)
    assert np.array_equal(n_neigh, want_nn)


def test_device_check_rejects_out_of_range_indices():
    """The device-side check of pp_create_crack (the host wrapper never
    passes such an index): nothing changes and IndexError is raised."""
    import torch
    from probabilistic_peridynamics_gb300.integrators import CUDAContext
    from probabilistic_peridynamics_gb300.neighbours import crack_device
    _, nlist, n_neigh = crack_cases(2)
    ctx = CUDAContext(0)
    nl = torch.as_tensor(nlist, device=ctx.device)
    nn = torch.as_tensor(n_neigh, device=ctx.device)
    n = nlist.shape[0]
    c = torch.tensor([[0, 1], [2, n]], dtype=torch.int32, device=ctx.device)
    with pytest.raises(IndexError):
        crack_device(c, nl, nn, ctx)
    assert np.array_equal(nl.cpu().numpy(), nlist)
    assert np.array_equal(nn.cpu().numpy(), n_neigh)


def test_empty_crack_list():
    _, nlist, n_neigh = crack_cases(3)
    nl, nn = nlist.copy(), n_neigh.copy()
    _gpu(np.zeros((0, 2), dtype=np.intc), nl, nn)
    assert np.array_equal(nl, nlist) and np.array_equal(nn, n_neigh)


def test_model_cuts_initial_crack_on_gpu(golden, tmp_path):
    """Model(..., initial_crack=...) with a CUDA integrator: the crack of
    the reference regression setup.  The counts and the neighbour sets
    equal the reference's golden (whose rows are in KD-tree order, ours
    ascending); the layout equals the sequential crack of the same rows."""
    import probabilistic_peridynamics_gb300 as pp
    from probabilistic_peridynamics_gb300.mesh import write_vtk
    from probabilistic_peridynamics_gb300.neighbours import neighbour_family
    from tests.plate_setup import crack_pairs, is_crack
    mesh = tmp_path / "plate.vtk"
    write_vtk(mesh, golden["points"], [("triangle", golden["cells_triangle"]),
                                       ("line", golden["cells_line"])])
    integ = pp.EulerCUDA(dt=1e-3)
    model = pp.Model(mesh, integrator=integ, horizon=0.1,
                     critical_stretch=0.005, bond_stiffness=1.0,
                     initial_crack=pp.initial_crack_helper(is_crack))
    nlist, n_neigh = model.initial_connectivity
    assert np.array_equal(n_neigh, golden["euler_n_neigh"])
    for i in range(nlist.shape[0]):
        assert np.array_equal(np.sort(nlist[i, :n_neigh[i]]),
                              np.sort(golden["euler_nlist"][i, :n_neigh[i]]))
    family, rows, _ = neighbour_family(golden["points"], 0.1, integ.context)
    counts = family.copy()
    crack = np.array(crack_pairs(golden["points"], rows, counts),
                     dtype=np.intc)
    _sequential()(crack, rows, counts)
    assert np.array_equal(nlist, rows) and np.array_equal(n_neigh, counts)
