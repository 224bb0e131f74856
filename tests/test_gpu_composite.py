"""Irregular two-material composite with trilinear damage (GPU).

The composite workload (Poisson-disk points, bond types 0/1/2 with the
interface at the harmonic-mean micro-modulus, three regimes per type) at a
size the oracle steps in seconds: 2,500 points in 0.16 x 0.08 x 0.04 (the
point density of 1M points in 2.0 x 1.0 x 0.1), Velocity-Verlet, dt 1e-6,
faces pulled 3e-6 per step for 200 steps: bonds move through all three
regimes, back down, and break.

Bars: FP64 paths bit-identical to the oracle (state, regimes, neighbour
list).  Mixed path, with and without compensated force sums: the same
broken-bond mask, regimes and intact counts as the oracle at steps 100 and
200; displacement error below 1e-5 of max|u| at step 100 (breaking has
begun); at step 200 below 1e-5 times the amplification A that the
problem itself applies between steps 100 and 200 to a perturbation of the
FP64 run (initial velocities perturbed by 3e-12 m/s, A measured in the
test: ~40).  Softening bonds (regime 2, negative stiffness) and fracture
amplify any difference: the mixed error grows from 4e-7 to 1.6e-5 over
those steps, as the perturbation of the FP64 run does.  Compensated sums
change the error by under 1%: the FP32 rounding of each bond force, not
the summation, sets it.
"""
import numpy as np
import pytest

from oracle import cl_step
from tests.conftest import cuda_available
from tests.gpu_helpers import rel_err

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]

MIXED_TOL = 1e-5
STEPS = 200
DT = 1e-6
RATE = 3e-6
DAMPING = 2.5e6


@pytest.fixture(scope="module")
def workload():
    from probabilistic_peridynamics_gb300.pointset import composite
    w = composite(count=2500, box=(0.16, 0.08, 0.04), split=0.08, seed=2)
    n = w["coords"].shape[0]
    w.update(nnodes=n, force_bc_types=np.zeros((n, 3), dtype=np.intc),
             force_bc_values=np.zeros((n, 3)), dt=DT)
    return w


@pytest.fixture(scope="module")
def oracle_run(workload):
    w = workload
    st = cl_step.Stepper(
        "velocity_verlet", DT, w["coords"], w["volume"], w["family"],
        w["nlist"], w["bc_types"], w["bc_values"], w["force_bc_types"],
        w["force_bc_values"], w["bond_stiffness"], w["critical_stretch"],
        damping=DAMPING, densities=w["densities"],
        bond_types=w["bond_types"], plus_cs=w["plus_cs"],
        nregimes=w["nregimes"])
    for k in range(STEPS):
        st.step(RATE * (k + 1), 0.0)
    return st.write(), st.regimes.copy()


def _run(w, checkpoints=(STEPS,), ud0=None, **kw):
    """States (``write()`` tuple, regimes) at each checkpoint step."""
    import probabilistic_peridynamics_gb300 as pp
    integ = pp.VelocityVerletCUDA(damping=DAMPING, dt=DT, **kw)
    n = w["nnodes"]
    integ.build(n, 3, w["max_neigh"], w["coords"], w["volume"], w["family"],
                w["bc_types"], w["bc_values"], w["force_bc_types"],
                w["force_bc_values"], None, w["bond_types"], w["densities"])
    z = lambda: np.zeros((n, 3))  # noqa: E731
    integ.create_buffers(w["nlist"].copy(), w["n_neigh"].copy(),
                         w["bond_stiffness"], w["critical_stretch"],
                         w["plus_cs"], z(), z() if ud0 is None else ud0, z(),
                         z(), z(), np.zeros(n), None, w["nregimes"],
                         w["nbond_types"])
    snaps = []
    for k in range(max(checkpoints)):
        integ(RATE * (k + 1), 0.0)
        if k + 1 in checkpoints:
            out = integ.write(z(), z(), z(), z(), z(), np.zeros(n),
                              w["nlist"].copy(), w["n_neigh"].copy())
            snaps.append((out, integ.regimes_d.cpu().numpy()))
    return snaps


def test_oracle_run_exercises_regimes_and_breaks(workload, oracle_run):
    (_, _, _, _, _, _, nlist, _), regimes = oracle_run
    broken = int((workload["nlist"] != -1).sum() - (nlist != -1).sum())
    assert broken > 100
    live = regimes[nlist != -1]
    assert np.any(live == 1) and np.any(live == 2)
    # all three bond types still carry intact bonds
    assert set(np.unique(workload["bond_types"][nlist != -1])) == {0, 1, 2}


@pytest.mark.parametrize("fused", [False, True], ids=["plain", "fused64"])
def test_fp64_bit_identical(workload, oracle_run, fused):
    [(out, regimes)] = _run(workload, fused=fused)
    ref, ref_regimes = oracle_run
    for got, want in zip(out, ref):
        assert np.array_equal(got, want)
    assert np.array_equal(regimes, ref_regimes)


@pytest.fixture(scope="module")
def fp64_runs(workload):
    """FP64 states at steps 100 and 200 (bit-identical to the oracle), and
    the amplification of a 3e-12 m/s velocity perturbation between them."""
    base = _run(workload, (100, 200))
    rng = np.random.default_rng(0)
    pert = _run(workload, (100, 200),
                ud0=3e-12 * rng.standard_normal((workload["nnodes"], 3)))
    e = [rel_err(p[0][0], b[0][0]) for p, b in zip(pert, base)]
    return base, e[1] / e[0]


@pytest.mark.parametrize("compensated", [False, True],
                         ids=["fp32sum", "compensated"])
def test_mixed_within_tolerance(workload, oracle_run, fp64_runs,
                                compensated):
    base, amplification = fp64_runs
    ref, ref_regimes = oracle_run
    assert np.array_equal(base[1][0][0], ref[0])  # the FP64 run is the oracle's
    snaps = _run(workload, (100, 200), precision="mixed",
                 compensated=compensated)
    for (out, regimes), (want, want_regimes) in zip(snaps, base):
        live = want[6] != -1
        assert int((out[6] != want[6]).sum()) == 0
        assert np.array_equal(regimes[live], want_regimes[live])
        assert np.array_equal(out[7], want[7])
    assert rel_err(snaps[0][0][0], base[0][0][0]) < MIXED_TOL
    assert rel_err(snaps[1][0][0], base[1][0][0]) < \
        MIXED_TOL * max(1.0, amplification)
