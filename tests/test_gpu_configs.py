"""The plain-method workloads at their stated sizes (GPU).

* 20x20x5 lattice, dx 0.05, horizon 3.015 dx, PMB with K = 1e9 and
  s0 = 0.005, x faces pulled apart 1e-8 per step, Euler dt = 1e-6, 1000
  steps, FP64: as stated the explicit step is unstable (the Euler update
  u += dt f needs dt < 2 / lambda_max, lambda_max <= 2 sum_j c vol / |xi_j|
  ~ 3e12 here, so dt lambda_max ~ 3e6): displacements grow until most
  bonds break.  The plain and fused FP64 steps still reproduce the oracle
  bit for bit through the blow-up (NaN where the oracle has NaN).  A stable
  labelled variant (dt = 1e-13, dt lambda_max ~ 0.3) is held to the usual
  bars: FP64 bit-identical, mixed within 1e-5 with the same mask.  The
  same workload through PeriPy's CPU integrator (``Euler``, on the GPU) is
  bit-identical to the reference's compiled Cython step, as stated and
  stable.
* 200x200x10 pre-cracked lattice (400,000 nodes, 42.7M bonds),
  Velocity-Verlet: at this size the oracle is too slow, so the FP64 fused
  step is checked against the plain FP64 step (each pinned to the oracle at
  small sizes) bit for bit over 10 steps, and the mixed step against the
  fused FP64 step over 300 steps (error < 1e-5, same mask).
"""
import numpy as np
import pytest

from tests.conftest import cuda_available
from tests.gpu_helpers import rel_err, run_integrator

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]


def _small(dt):
    from probabilistic_peridynamics_gb300 import lattice
    coords = lattice.lattice_coords(20, 20, 5, 0.05)
    family, nlist, width = lattice.lattice_family(20, 20, 5, 3.015)
    bc_types, bc_values = lattice.face_bcs(coords, 0)
    n = coords.shape[0]
    return dict(coords=coords, volume=np.full(n, 0.05 ** 3), family=family,
                nlist=nlist, n_neigh=family.copy(), bc_types=bc_types,
                bc_values=bc_values,
                force_bc_types=np.zeros((n, 3), dtype=np.intc),
                force_bc_values=np.zeros((n, 3)), nnodes=n,
                max_neigh=int(width),
                k=lattice.bond_stiffness_pmb(1e9, 3.015 * 0.05), s0=0.005,
                dt=dt)


def _oracle(setup, steps, mags):
    from oracle import cref
    st = cref.Stepper("euler", setup["dt"], setup["coords"], setup["volume"],
                      setup["family"], setup["nlist"], setup["bc_types"],
                      setup["bc_values"], setup["force_bc_types"],
                      setup["force_bc_values"], setup["k"], setup["s0"])
    for k in range(steps):
        st.step(mags[k], 0.0)
    return st.write()


STEPS = 1000
MAGS = 1e-8 * np.arange(1, STEPS + 1)


@pytest.fixture(scope="module")
def stated_oracle():
    setup = _small(1e-6)
    return setup, _oracle(setup, STEPS, MAGS)


@pytest.mark.parametrize("fused", [False, True], ids=["plain", "fused64"])
def test_small_lattice_as_stated(stated_oracle, fused):
    import probabilistic_peridynamics_gb300 as pp
    setup, ref = stated_oracle
    assert family_sum(setup) == 166_508
    # the stated step is unstable: the oracle itself blows up
    assert not np.all(np.isfinite(ref[0])) or np.abs(ref[0]).max() > 1.0
    out = run_integrator(pp.EulerCUDA(dt=setup["dt"], fused=fused), setup,
                         STEPS, MAGS)
    for got, want in zip(out, ref):
        assert np.array_equal(got, want, equal_nan=True)


def family_sum(setup):
    return int(setup["family"].sum())


@pytest.mark.parametrize("mode", ["plain", "fused64", "mixed"])
def test_small_lattice_stable_variant(mode):
    import probabilistic_peridynamics_gb300 as pp
    setup = _small(1e-13)
    ref = _oracle(setup, STEPS, MAGS)
    assert np.all(np.isfinite(ref[0]))
    integ = pp.EulerCUDA(dt=setup["dt"], fused=mode != "plain",
                         precision="mixed" if mode == "mixed" else "float64")
    out = run_integrator(integ, setup, STEPS, MAGS)
    if mode == "mixed":
        assert np.array_equal(out[6], ref[6])
        assert rel_err(out[0], ref[0]) < 1e-5
    else:
        for got, want in zip(out, ref):
            assert np.array_equal(got, want)


@pytest.mark.parametrize("dt", [1e-6, 1e-13], ids=["as_stated", "stable"])
def test_small_lattice_cpu_integrator(dt):
    """The plain method's own CPU integrator (``Euler``, the Cython step)
    on the small lattice, 1000 steps, through the GPU ``Euler``: bit for
    bit the reference's compiled ``peridynamics.pyx`` on the same compact
    rows, through the blow-up of the stated dt as well."""
    from oracle import build_ref
    from probabilistic_peridynamics_gb300 import lattice
    from tests.cython_setup import run_gpu_euler, run_reference_euler
    if not build_ref.build(quiet=True):
        pytest.skip("the compiled reference is not available")
    ref = build_ref.load()
    setup = _small(dt)
    family, nlist, _ = lattice.lattice_family(20, 20, 5, 3.015, pow2=False)
    nlist = np.where(nlist == -1, 0, nlist).astype(np.intc)  # 0-padded
    setup = dict(setup, family=family, nlist=nlist, n_neigh=family.copy())
    args = (setup, STEPS, MAGS, dt, setup["k"], setup["s0"])
    with np.errstate(all="ignore"):
        want = run_reference_euler(ref, *args)
    got = run_gpu_euler(*args)
    for g, w in zip(got, want):
        assert np.array_equal(g, w, equal_nan=True)
    broken = int(family.sum() - want[4].sum())
    if dt == 1e-6:
        assert broken > 1000  # the unstable step breaks bonds (|strain|)
    else:
        assert broken == 0 and np.all(np.isfinite(want[0]))


@pytest.fixture(scope="module")
def large():
    import bench
    return bench.build_workload()


def _large_run(w, precision, fused, steps):
    import bench
    integ = bench.make_integrator(w, precision, fused, autotune=False)
    mags = bench.PULL_RATE * np.arange(1, steps + 1)
    if fused:
        integ._run(mags, np.zeros(steps), 0, steps)
    else:
        for k in range(steps):
            integ(mags[k], 0.0)
    n = w["nnodes"]
    z = [np.zeros((n, 3)) for _ in range(5)]
    return integ.write(*z, np.zeros(n), w["nlist"].copy(), w["n_neigh"].copy())


def test_large_lattice_fused_fp64_equals_plain(large):
    assert large["bonds"] == 42_700_528 and large["nnodes"] == 400_000
    a = _large_run(large, "float64", False, 10)
    b = _large_run(large, "float64", True, 10)
    for got, want in zip(b, a):
        assert np.array_equal(got, want)


def test_large_lattice_mixed_vs_fp64(large):
    ref = _large_run(large, "float64", True, 300)
    out = _large_run(large, "mixed", True, 300)
    assert np.array_equal(out[6], ref[6])
    assert np.array_equal(out[7], ref[7])
    assert rel_err(out[0], ref[0]) < 1e-5
