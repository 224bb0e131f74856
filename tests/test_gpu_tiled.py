"""The tiled layout of the mixed step against the untiled kernel (GPU).

On rows without holes (every neighbour list ``Model`` builds, cracked or
not) the tiled kernel sums each node's bonds in the order the untiled kernel
does for rows of 64 slots or more (lane l of eight takes row entries l,
l + 8, ...; the same FP32 bond arithmetic on the same exact bond vectors;
the same reduction), so the two are bit for bit identical: positions,
velocities, accelerations, forces, the broken-bond mask, intact counts and
regimes.  That holds for any internal ordering and any cut into tiles,
including tiles whose halo overflows the capacity and is split, and a
random ordering with one-node tiles.
"""
import numpy as np
import pytest

from tests.conftest import cuda_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]


def _run(cls_args, w, steps, mags, tiled, u0=None, order=None,
         halo_cap=None, monkeypatch=None, types=False, compensated=False,
         instances=None, corrections=None, variant=None):
    from probabilistic_peridynamics_gb300 import tiling
    cls, args = cls_args
    integ = cls(*args, precision="mixed", tiled=tiled, autotune=False,
                compensated=compensated)
    if instances is not None:
        integ.set_instances(*instances)
    n = w["nnodes"]
    integ.build(n, 3, w["max_neigh"], w["coords"], w["volume"], w["family"],
                w["bc_types"], w["bc_values"], w["force_bc_types"],
                w["force_bc_values"], corrections,
                w.get("bond_types") if types else None, w.get("densities"))
    if order is not None:
        integ._order = order
    if halo_cap is not None:
        monkeypatch.setattr(tiling, "HALO_CAP", halo_cap)
    z = np.zeros((n, 3))
    if types:
        integ.create_buffers(w["nlist"], w["n_neigh"], w["bond_stiffness"],
                             w["critical_stretch"], w["plus_cs"],
                             z if u0 is None else u0, z, z, z, z,
                             np.zeros(n), None, w["nregimes"],
                             w["nbond_types"])
    else:
        integ.create_buffers(w["nlist"], w["n_neigh"], w["k"], w["s0"], None,
                             z if u0 is None else u0, z, z, z, z,
                             np.zeros(n), None, 1, 1)
    if variant is not None:
        integ._fargs.variant = variant
    integ._run(mags, np.zeros(steps), 0, steps)
    zz = [np.zeros((n, 3)) for _ in range(5)]
    out = integ.write(*zz, np.zeros(n), w["nlist"].copy(),
                      w["n_neigh"].copy())
    regimes = (integ.regimes_d.cpu().numpy().copy()
               if integ.regimes_d is not None else None)
    stats = integ.tiling.stats() if integ.tiling is not None else None
    return out, regimes, stats


def _same(a, b):
    for x, y in zip(a[0], b[0]):
        assert np.array_equal(x, y)
    if a[1] is not None:
        assert np.array_equal(a[1], b[1])


@pytest.fixture(scope="module")
def plate():
    import bench
    return bench.build_workload()


def _vv():
    import bench
    import probabilistic_peridynamics_gb300 as pp
    return pp.VelocityVerletCUDA, (bench.DAMPING, bench.DT)


def test_plate_fracture_tiled_equals_untiled(plate):
    import bench
    u0, mags = bench.fracture_state(plate)
    steps = 100
    ref = _run(_vv(), plate, steps, mags(steps), False, u0=u0)
    got = _run(_vv(), plate, steps, mags(steps), True, u0=u0)
    assert int(np.sum(plate["nlist"] != -1) - np.sum(got[0][6] != -1)) > \
        100_000
    st = got[2]
    assert st["tiles"] == 3200 and st["splits"] == 0
    assert st["halo_max"] <= 768
    _same(got, ref)


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_tile_shapes_identical(plate, variant):
    import bench
    u0, mags = bench.fracture_state(plate)
    steps = 30
    ref = _run(_vv(), plate, steps, mags(steps), False, u0=u0)
    got = _run(_vv(), plate, steps, mags(steps), True, u0=u0,
               variant=variant)
    _same(got, ref)


def test_split_halos_and_random_order(monkeypatch):
    """A halo capacity of 200 records forces splits down to small tiles;
    a random permutation with one-node tiles gives the largest halos per
    node.  Both equal the untiled kernel bit for bit."""
    import probabilistic_peridynamics_gb300 as pp
    from tests.gpu_helpers import breaking_setup
    w = breaking_setup("velocity_verlet", 14, 12, 6)
    cls = (pp.VelocityVerletCUDA, (0.5, 1.0))
    steps = 40
    mags = 3e-3 * np.arange(1, steps + 1)
    ref = _run(cls, w, steps, mags, False)
    got = _run(cls, w, steps, mags, True, halo_cap=200,
               monkeypatch=monkeypatch)
    assert got[2]["splits"] > 0 and got[2]["halo_max"] <= 200
    _same(got, ref)
    n = w["nnodes"]
    perm = np.random.default_rng(3).permutation(n).astype(np.int32)
    got = _run(cls, w, steps, mags, True,
               order=(perm, np.arange(n + 1, dtype=np.int32)))
    assert got[2]["tiles"] == n
    _same(got, ref)
    assert int(np.sum(w["nlist"] != -1) - np.sum(got[0][6] != -1)) > 0


@pytest.mark.parametrize("variant", [0, 1, 2])
@pytest.mark.parametrize("compensated", [False, True])
def test_composite_types_tiled_equals_untiled(compensated, variant):
    """Bond types, three regimes, softening and breaking (2,500-point
    composite, 200 steps), on every tile shape."""
    import probabilistic_peridynamics_gb300 as pp
    from probabilistic_peridynamics_gb300.pointset import composite
    w = composite(count=2500, box=(0.16, 0.08, 0.04), split=0.08, seed=2)
    n = w["coords"].shape[0]
    w.update(nnodes=n, force_bc_types=np.zeros((n, 3), dtype=np.intc),
             force_bc_values=np.zeros((n, 3)))
    cls = (pp.VelocityVerletCUDA, (2.5e6, 1e-6))
    steps = 200
    mags = 3e-6 * np.arange(1, steps + 1)
    ref = _run(cls, w, steps, mags, False, types=True,
               compensated=compensated)
    got = _run(cls, w, steps, mags, True, types=True,
               compensated=compensated, variant=variant)
    assert np.count_nonzero(got[1]) > 0
    _same(got, ref)


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_batched_instances_tiled_equals_untiled(variant):
    """Per-instance critical stretch and per-bond stiffness corrections
    (five uneven lattices, Euler-Cromer, breaking), on every tile shape."""
    import probabilistic_peridynamics_gb300 as pp
    from probabilistic_peridynamics_gb300 import batch
    inst = batch.uq_instances(count=5, seed=5, nx_range=(6, 10),
                              ny_range=(5, 8), nz=3, dx=1.0, s0_mean=0.02,
                              s0_sigma=0.2, density=50.0)
    b = batch.concatenate(inst)
    w = dict(nnodes=b.nnodes, max_neigh=b.max_neigh, coords=b.coords,
             volume=b.volume, family=b.family, bc_types=b.bc_types,
             bc_values=b.bc_values, force_bc_types=b.force_bc_types,
             force_bc_values=b.force_bc_values, densities=b.densities,
             nlist=b.nlist, n_neigh=b.n_neigh, k=0.01,
             s0=float(b.instance_s0[0]))
    cls = (pp.EulerCromerCUDA, (0.5, 1.0))
    steps = 60
    mags = 3e-3 * np.arange(1, steps + 1)
    args = dict(instances=(b.node_instance, b.instance_s0),
                corrections=b.stiffness_corrections)
    ref = _run(cls, w, steps, mags, False, **args)
    got = _run(cls, w, steps, mags, True, variant=variant, **args)
    assert int(np.sum(b.nlist != -1) - np.sum(got[0][6] != -1)) > 0
    _same(got, ref)


@pytest.mark.parametrize("field", ["halo_max", "split_mark", "tile_start"])
def test_bad_tile_reported(field, monkeypatch):
    """A tile whose counts exceed the kernel's limits (here set on the host
    after the set-up: a halo longer than PP_TILE_HALO_MAX; the set-up's
    mark of a tile to split, halo_cap + 1, on the last tile of a tiling
    with a small halo_cap; more than PP_TILE_NODES_MAX nodes) is skipped by
    the step's own bounds checks and reported as PP_STATUS_BAD_TILING;
    write() raises."""
    import probabilistic_peridynamics_gb300 as pp
    from probabilistic_peridynamics_gb300 import _lib, tiling
    from tests.gpu_helpers import breaking_setup
    w = breaking_setup("velocity_verlet", 14, 12, 6)
    integ = pp.VelocityVerletCUDA(0.5, 1.0, precision="mixed", tiled=True,
                                  autotune=False)
    n = w["nnodes"]
    integ.build(n, 3, w["max_neigh"], w["coords"], w["volume"], w["family"],
                w["bc_types"], w["bc_values"], w["force_bc_types"],
                w["force_bc_values"], None, None, w.get("densities"))
    z = np.zeros((n, 3))
    if field == "split_mark":
        monkeypatch.setattr(tiling, "HALO_CAP", 400)
    integ.create_buffers(w["nlist"], w["n_neigh"], w["k"], w["s0"], None,
                         z, z, z, z, z, np.zeros(n), None, 1, 1)
    t = integ.tiling
    if field == "halo_max":
        t.halo_count_d[0] = _lib.PP_TILE_HALO_MAX + 1
    elif field == "split_mark":
        assert t.halo_cap == 400 < _lib.PP_TILE_HALO_MAX
        t.halo_count_d[t.struct.ntiles - 1] = t.halo_cap + 1
    else:
        # the first tile's end moved past PP_TILE_NODES_MAX nodes
        t.tile_start_d[1] = t.tile_start_d[0] + _lib.PP_TILE_NODES_MAX + 1
    integ(0.0, 0.0)
    zz = [np.zeros((n, 3)) for _ in range(5)]
    with pytest.raises(_lib.LibraryError, match="device status 2"):
        integ.write(*zz, np.zeros(n), w["nlist"].copy(), w["n_neigh"].copy())
