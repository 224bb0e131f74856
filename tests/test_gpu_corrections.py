"""Stiffness correction factors on the GPU (pp_stiffness_corrections).

Bar: bit-identical to the reference's own correction functions
(``peripy/correction.pyx``, compiled from the reference sources into
``oracle/_ref``), applied in the order and with the arguments
``peripy/model.py:349-375`` uses, on the pre-cracked 2113-node plate and on
a lattice whose neighbour list has one-sided removals; and through
``Model(..., micromodulus_function=..., volume_correction=...,
surface_correction=...)``.
"""
import numpy as np
import pytest

from tests.conftest import cuda_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]


@pytest.fixture(scope="module")
def ref():
    from oracle import build_ref
    if not build_ref.available():
        build_ref.build(quiet=True)
    if not build_ref.available():
        pytest.skip("reference correction module not built")
    return build_ref.load("correction")


def _reference(ref, coords, volume, nlist, n_neigh, horizon, mm, vc, sc,
               node_radius, dimensions=3):
    """The reference Model's sequence (model.py:349-375, 782-935)."""
    n, width = nlist.shape
    out = np.ones((n, width))
    search = horizon + node_radius if vc is not None else horizon
    if mm is not None:
        ref.set_micromodulus_function(out, coords, nlist, n_neigh,
                                      np.float64(horizon), np.intc(mm))
    if vc is not None:
        # _set_volume_corrections(vc, out, node_radius, horizon), whose
        # signature is (vc, out, horizon, node_radius)
        ref.set_volume_correction(out, coords, nlist, n_neigh,
                                  np.float64(node_radius),
                                  np.float64(horizon), np.intc(vc))
    if sc is not None:
        bulk = (np.float64(np.pi * np.power(search, 2)) if dimensions == 2
                else np.float64((4. / 3) * np.pi * np.power(search, 3)))
        if sc == 1:
            ref.set_precise_surface_correction(out, nlist, n_neigh, volume,
                                               bulk)
        else:
            ref.set_imprecise_surface_correction(
                out, nlist, n_neigh, np.float64(np.sum(volume) / n), bulk)
    return out


CASES = [(0, None, None), (None, 0, None), (None, None, 1),
         (None, None, 0), (0, 0, 1), (0, 0, 0)]


@pytest.fixture(scope="module")
def plate(golden):
    from tests.plate_setup import HORIZON, plate_inputs
    p = plate_inputs(golden)
    return p, HORIZON


@pytest.mark.parametrize("mm,vc,sc", CASES)
def test_plate_matches_reference(ref, plate, mm, vc, sc):
    from probabilistic_peridynamics_gb300.corrections import \
        stiffness_corrections
    p, horizon = plate
    nr = 0.02
    nlist = np.ascontiguousarray(p["nlist"], dtype=np.intc)
    n_neigh = np.ascontiguousarray(p["n_neigh"], dtype=np.intc)
    want = _reference(ref, p["coords"], p["volume"], nlist, n_neigh,
                      horizon, mm, vc, sc, nr, dimensions=2)
    got = stiffness_corrections(
        p["coords"], p["volume"], nlist, n_neigh, horizon,
        micromodulus_function=mm, volume_correction=vc,
        surface_correction=sc, node_radius=nr, dimensions=2,
        search_horizon=horizon + nr if vc is not None else horizon)
    assert np.array_equal(got, want)
    assert not np.all(got == 1.0)


def test_one_sided_removals_match_reference(ref):
    """Slots whose reverse bond is missing follow the reference's pair
    visit: a slot (i -> j), j < i, is corrected only when j's row holds i."""
    from probabilistic_peridynamics_gb300 import lattice
    from probabilistic_peridynamics_gb300.corrections import \
        stiffness_corrections
    coords = lattice.lattice_coords(8, 6, 5, 0.1)
    family, nlist, _ = lattice.lattice_family(8, 6, 5, 3.015)
    n_neigh = family.copy()
    rng = np.random.default_rng(1)
    # remove j from i's row only (swap-remove, rows stay compact)
    for i in rng.choice(coords.shape[0], 40, replace=False):
        k = int(rng.integers(n_neigh[i]))
        nlist[i, k] = nlist[i, n_neigh[i] - 1]
        nlist[i, n_neigh[i] - 1] = -1
        n_neigh[i] -= 1
    volume = rng.uniform(0.8e-3, 1.2e-3, coords.shape[0])
    for mm, vc, sc in CASES:
        want = _reference(ref, coords, volume, nlist, n_neigh, 0.3015, mm,
                          vc, sc, 0.05)
        got = stiffness_corrections(
            coords, volume, nlist, n_neigh, 0.3015, micromodulus_function=mm,
            volume_correction=vc, surface_correction=sc, node_radius=0.05,
            search_horizon=0.3515 if vc is not None else 0.3015)
        assert np.array_equal(got, want), (mm, vc, sc)


def test_flags_checked_like_the_reference():
    from probabilistic_peridynamics_gb300.corrections import \
        stiffness_corrections
    z = np.zeros((2, 3))
    nl = np.array([[1], [0]], dtype=np.intc)
    nn = np.ones(2, dtype=np.intc)
    assert stiffness_corrections(z, np.ones(2), nl, nn, 1.0) is None
    with pytest.raises(ValueError):
        stiffness_corrections(z, np.ones(2), nl, nn, 1.0,
                              micromodulus_function=1)
    with pytest.raises(ValueError):
        stiffness_corrections(z, np.ones(2), nl, nn, 1.0,
                              surface_correction=2)


def test_model_builds_the_corrections(ref, golden, tmp_path):
    """Model(...) with the three flags: the factors of the reference
    sequence on the Model's own connectivity."""
    import probabilistic_peridynamics_gb300 as pp
    from probabilistic_peridynamics_gb300.mesh import write_vtk
    from tests.plate_setup import HORIZON
    coords = golden["points"]
    mesh = tmp_path / "plate.vtk"
    write_vtk(mesh, coords, [("triangle", golden["cells_triangle"]),
                             ("line", golden["cells_line"])])
    nr = 0.01
    model = pp.Model(mesh, integrator=pp.EulerCUDA(dt=1e-3),
                     horizon=HORIZON, critical_stretch=0.005,
                     bond_stiffness=1.0, micromodulus_function=0,
                     volume_correction=0, surface_correction=1,
                     node_radius=nr)
    nlist, n_neigh = model.initial_connectivity
    want = _reference(ref, model.coords, model.volume,
                      np.ascontiguousarray(nlist, dtype=np.intc),
                      np.ascontiguousarray(n_neigh, dtype=np.intc), HORIZON,
                      0, 0, 1, nr, dimensions=2)
    assert np.array_equal(model.stiffness_corrections, want)
