"""The workloads at their stated sizes against the CPU oracle (GPU).

The C restatement of the OpenCL step (``oracle/pp_oracle.c``, OpenMP over
nodes, bit-identical to the NumPy oracle and pinned to the reference's
goldens) steps every one of these in well under a second, so the binary64
CUDA step is compared with it bit for bit at full size, and the mixed step
with the binary64 one where bonds break.

* Plate (200 x 200 x 10, 400,000 nodes, 42.7M bonds, pre-cracked,
  Velocity-Verlet), fracture variant: released at rest from a uniform
  strain of 0.004 along x (80 % of s0), faces held at that strain and pulled
  on.  Bonds start breaking after a few steps (23,612 by step 20, about
  270,000 by step 100, 380,000 by step 300).  FP64 fused = oracle bit for
  bit over 20 steps; mixed vs FP64 over 300 steps: 0 mask flips, equal
  intact counts, displacement error < 1e-5 (peridynamics.cl:78-91 break
  semantics: -1 written into the neighbour list).
* Batched UQ (64 instances, 4,996,875 nodes, 461M bonds, Euler-Cromer,
  per-instance s0, per-bond stiffness noise): as stated (from rest, faces
  pulled 1e-8 per step) and pre-strained to 80 % of each instance's own s0;
  20 steps each.  The smallest and the largest instance of the batched FP64
  run equal the oracle run on that instance alone bit for bit; every
  instance of the mixed run has the FP64 run's mask and is within 1e-5.
* Composite (1M Poisson-disk points, three bond types, trilinear damage,
  Velocity-Verlet): FP64 fused = oracle bit for bit over 10 steps from a
  strain of 0.0045 (above the first regime threshold, so regimes change
  from the first step); mixed with compensated sums vs FP64 as stated
  (from rest, faces pulled 5e-7 per step) over 200 steps: identical mask
  and regimes, error < 1e-5.  Through softening and fracture (strain 0.0035:
  62k bonds broken and 345k softened by step 100) the problem amplifies
  any perturbation; there the mixed run keeps the FP64 mask, differs in
  the regime of at most 1e-4 of the softened bonds (a bond at a threshold
  switching a step apart), and its error grows no faster than that of an
  FP64 run whose initial velocities are perturbed by 3e-12 m/s.
"""
import numpy as np
import pytest

from tests.conftest import cuda_available
from tests.gpu_helpers import rel_err

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]

ARRAYS = ("u", "ud", "udd", "force", "body_force", "damage", "nlist",
          "n_neigh")


def _free():
    import torch
    torch.cuda.empty_cache()


def _write(integ, n, nlist, n_neigh):
    z = [np.zeros((n, 3)) for _ in range(5)]
    return integ.write(*z, np.zeros(n), nlist.copy(), n_neigh.copy())


def _assert_identical(got, want):
    for name, g, w in zip(ARRAYS, got, want):
        assert np.array_equal(g, w), name


# ------------------------------------------------------------------ plate
@pytest.fixture(scope="module")
def plate():
    import bench
    return bench.build_workload()


def test_plate_fp64_matches_c_oracle_through_fracture(plate):
    import bench
    from oracle import cref
    w = plate
    u0, mags = bench.fracture_state(w)
    steps = 20
    m = mags(steps)
    st = cref.Stepper("velocity_verlet", bench.DT, w["coords"], w["volume"],
                      w["family"], w["nlist"], w["bc_types"], w["bc_values"],
                      w["force_bc_types"], w["force_bc_values"], w["k"],
                      w["s0"], damping=bench.DAMPING,
                      densities=w["densities"])
    st.u[:] = u0
    for k in range(steps):
        st.step(m[k], 0.0)
    want = st.write()
    integ = bench.make_integrator(w, "float64", True, autotune=False, u0=u0)
    integ._run(m, np.zeros(steps), 0, steps)
    got = _write(integ, w["nnodes"], w["nlist"], w["n_neigh"])
    del integ
    _free()
    broken = int(np.sum(w["nlist"] != -1) - np.sum(want[6] != -1))
    assert broken > 10_000
    _assert_identical(got, want)


def test_plate_fracture_mixed_vs_fp64(plate):
    import bench
    res = bench.accuracy_fracture(plate, __import__("torch"),
                                  checkpoints=(100, 300))
    for c in (100, 300):
        r = res[f"step_{c}"]
        assert r["bonds_broken_fp64"] > 100_000, r
        assert r["mask_flips_vs_fp64"] == 0, r
        assert r["n_neigh_equal"], r
        assert r["disp_rel_err_vs_fp64"] < 1e-5, r


# ---------------------------------------------------------------- batched
@pytest.fixture(scope="module")
def uq():
    import bench
    from probabilistic_peridynamics_gb300 import batch, lattice
    inst = batch.uq_instances(count=64, seed=2024, dx=bench.DX)
    b = batch.concatenate(inst)
    k = lattice.bond_stiffness_pmb(bench.BULK_MODULUS,
                                   bench.HORIZON_CELLS * bench.DX)
    return inst, b, k


def _prestrain(inst, b, frac):
    """Each instance at ``frac`` of its own critical stretch along x; its x
    faces hold that displacement (scaled by the magnitude)."""
    u0 = np.zeros((b.nnodes, 3))
    bcv = b.bc_values.copy()
    for kk, ins in enumerate(inst):
        a, e = b.offsets[kk], b.offsets[kk + 1]
        x = b.coords[a:e, 0]
        u0[a:e, 0] = frac * ins.critical_stretch * (x - 0.5 * (x.min() +
                                                               x.max()))
        face = b.bc_types[a:e, 0] != 0
        bcv[a:e, 0] = np.where(face, u0[a:e, 0], 0.0)
    return u0, bcv


def _batch_run(b, k, precision, mags, u0=None, bcv=None):
    import bench
    import probabilistic_peridynamics_gb300 as pp
    integ = pp.EulerCromerCUDA(bench.DAMPING, dt=bench.DT,
                               precision=precision, autotune=False)
    integ.set_instances(b.node_instance, b.instance_s0)
    integ.build(b.nnodes, 3, b.max_neigh, b.coords, b.volume, b.family,
                b.bc_types, b.bc_values if bcv is None else bcv,
                b.force_bc_types, b.force_bc_values, b.stiffness_corrections,
                None, b.densities)
    z = np.zeros((b.nnodes, 3))
    integ.create_buffers(b.nlist, b.n_neigh, k, float(b.instance_s0[0]),
                         None, z if u0 is None else u0, z, z, z, z,
                         np.zeros(b.nnodes), None, 1, 1)
    integ._run(mags, np.zeros(len(mags)), 0, len(mags))
    out = _write(integ, b.nnodes, b.nlist, b.n_neigh)
    del integ
    _free()
    return out


def _instance_oracle(ins, k, mags, u0=None, bcv=None):
    import bench
    from oracle import cref
    n = ins.nnodes
    st = cref.Stepper("euler_cromer", bench.DT, ins.coords, ins.volume,
                      ins.family, ins.nlist, ins.bc_types,
                      ins.bc_values if bcv is None else bcv,
                      np.zeros((n, 3), dtype=np.intc), np.zeros((n, 3)), k,
                      ins.critical_stretch, damping=bench.DAMPING,
                      densities=ins.densities,
                      stiffness_corrections=ins.stiffness_corrections)
    if u0 is not None:
        st.u[:] = u0
    for m in mags:
        st.step(m, 0.0)
    return st.write()


@pytest.mark.parametrize("loading", ["as_stated", "prestrained"])
def test_batched_uq_full_size(uq, loading):
    import bench
    inst, b, k = uq
    assert len(inst) == 64 and b.bonds > 4e8
    steps = 20
    if loading == "as_stated":
        u0 = bcv = None
        mags = bench.PULL_RATE * np.arange(1, steps + 1)
    else:
        u0, bcv = _prestrain(inst, b, 0.8)
        mags = 1.0 + 1e-4 * np.arange(1, steps + 1)
    r64 = _batch_run(b, k, "float64", mags, u0, bcv)
    r32 = _batch_run(b, k, "mixed", mags, u0, bcv)
    sizes = [ins.nnodes for ins in inst]
    broken = 0
    for kk in (int(np.argmin(sizes)), int(np.argmax(sizes))):
        a, e = b.offsets[kk], b.offsets[kk + 1]
        ins = inst[kk]
        want = _instance_oracle(ins, k, mags,
                                None if u0 is None else u0[a:e],
                                None if bcv is None else bcv[a:e])
        w = ins.nlist.shape[1]
        nl = np.where(r64[6][a:e, :w] >= 0, r64[6][a:e, :w] - a, -1)
        assert np.array_equal(nl, want[6])
        assert np.array_equal(r64[7][a:e], want[7])
        for g, ref in zip(r64[:6], want[:6]):
            assert np.array_equal(g[a:e], ref)
        broken += int(np.sum(ins.nlist != -1) - np.sum(want[6] != -1))
    assert np.array_equal(r32[6], r64[6])
    assert np.array_equal(r32[7], r64[7])
    for kk in range(len(inst)):
        a, e = b.offsets[kk], b.offsets[kk + 1]
        assert rel_err(r32[0][a:e], r64[0][a:e]) < 1e-5, kk
    if loading == "prestrained":
        assert broken > 0
        assert int(np.sum(b.nlist != -1) - np.sum(r64[6] != -1)) > 10_000


# -------------------------------------------------------------- composite
COMPOSITE_DT = 1e-6
COMPOSITE_DAMPING = 2.5e6
COMPOSITE_RATE = 5e-7


@pytest.fixture(scope="module")
def composite_1m():
    from probabilistic_peridynamics_gb300.integrators import CUDAContext
    from probabilistic_peridynamics_gb300.pointset import composite
    w = composite(context=CUDAContext(0))
    n = w["coords"].shape[0]
    w.update(nnodes=n, force_bc_types=np.zeros((n, 3), dtype=np.intc),
             force_bc_values=np.zeros((n, 3)))
    return w


def _composite_u0(w, eps0):
    x = w["coords"][:, 0]
    u0 = np.zeros((w["nnodes"], 3))
    u0[:, 0] = eps0 * (x - 1.0)
    return u0, eps0 * (x.max() - 1.0)


def _composite_run(w, precision, mags, checkpoints, u0=None, ud0=None,
                   compensated=False):
    """``{step: (write tuple, regimes)}``."""
    import probabilistic_peridynamics_gb300 as pp
    n = w["nnodes"]
    integ = pp.VelocityVerletCUDA(COMPOSITE_DAMPING, dt=COMPOSITE_DT,
                                  precision=precision,
                                  compensated=compensated, autotune=False)
    integ.build(n, 3, w["max_neigh"], w["coords"], w["volume"], w["family"],
                w["bc_types"], w["bc_values"], w["force_bc_types"],
                w["force_bc_values"], None, w["bond_types"], w["densities"])
    z = np.zeros((n, 3))
    integ.create_buffers(w["nlist"], w["n_neigh"], w["bond_stiffness"],
                         w["critical_stretch"], w["plus_cs"],
                         z if u0 is None else u0, z if ud0 is None else ud0,
                         z, z, z, np.zeros(n), None, w["nregimes"],
                         w["nbond_types"])
    out, done = {}, 0
    for c in checkpoints:
        integ._run(mags, np.zeros(len(mags)), done, c - done)
        done = c
        res = _write(integ, n, w["nlist"], w["n_neigh"])
        out[c] = (res, integ.regimes_d.cpu().numpy().copy())
    del integ
    _free()
    return out


def test_composite_fp64_matches_c_oracle(composite_1m):
    from oracle import cref
    w = composite_1m
    u0, face = _composite_u0(w, 0.0045)
    steps = 10
    mags = face + COMPOSITE_RATE * np.arange(1, steps + 1)
    st = cref.Stepper("velocity_verlet", COMPOSITE_DT, w["coords"],
                      w["volume"], w["family"], w["nlist"], w["bc_types"],
                      w["bc_values"], w["force_bc_types"],
                      w["force_bc_values"], w["bond_stiffness"],
                      w["critical_stretch"], damping=COMPOSITE_DAMPING,
                      densities=w["densities"], bond_types=w["bond_types"],
                      plus_cs=w["plus_cs"], nregimes=w["nregimes"])
    st.u[:] = u0
    for m in mags:
        st.step(m, 0.0)
    want = st.write()
    (got, regimes), = _composite_run(w, "float64", mags, (steps,),
                                     u0=u0).values()
    assert np.count_nonzero(st.regimes) > 100_000
    assert np.array_equal(regimes, st.regimes)
    _assert_identical(got, want)


def test_composite_mixed_as_stated(composite_1m):
    w = composite_1m
    steps = 200
    mags = COMPOSITE_RATE * np.arange(1, steps + 1)
    (r64, g64), = _composite_run(w, "float64", mags, (steps,)).values()
    (r32, g32), = _composite_run(w, "mixed", mags, (steps,),
                                 compensated=True).values()
    assert np.array_equal(r32[6], r64[6])
    assert np.array_equal(g32, g64)
    assert np.array_equal(r32[7], r64[7])
    assert rel_err(r32[0], r64[0]) < 1e-5


def test_composite_mixed_through_softening(composite_1m):
    """Strain 0.0035: the broken-bond mask equals the FP64 run's at steps
    50 and 100.  The regime of a bond whose stretch sits within the state
    difference (~1e-7 relative) of a regime threshold can switch a step
    earlier or later than in the FP64 run: the regimes may differ for a
    handful of the hundreds of thousands of softened bonds, and the
    displacement error grows with the problem's own amplification of a
    perturbation (FP64 run with velocities perturbed by 3e-12 m/s)."""
    w = composite_1m
    u0, face = _composite_u0(w, 0.0035)
    steps = (50, 100)
    mags = face + COMPOSITE_RATE * np.arange(1, steps[-1] + 1)
    ref = _composite_run(w, "float64", mags, steps, u0=u0)
    pert = 3e-12 * np.random.default_rng(0).standard_normal((w["nnodes"], 3))
    per = _composite_run(w, "float64", mags, steps, u0=u0, ud0=pert)
    mix = _composite_run(w, "mixed", mags, steps, u0=u0, compensated=True)
    e_mix, e_per, stats = {}, {}, {}
    for c in steps:
        (r64, g64), (r32, g32) = ref[c], mix[c]
        valid = r64[6] != -1
        softened = int(np.count_nonzero(g64[valid]))
        e_mix[c] = rel_err(r32[0], r64[0])
        e_per[c] = rel_err(per[c][0][0], r64[0])
        stats[c] = dict(flips=int(np.sum(r32[6] != r64[6])),
                        regime_diff=int(np.sum(g32 != g64)),
                        regime_diff_perturbed=int(np.sum(per[c][1] != g64)),
                        softened=softened, err=e_mix[c],
                        err_perturbed=e_per[c])
    print("composite softening:", stats)
    broken = int(np.sum(w["nlist"] != -1) - np.sum(ref[100][0][6] != -1))
    assert broken > 10_000
    for c in steps:
        assert stats[c]["flips"] == 0, stats
        assert stats[c]["softened"] > 100_000, stats
        assert stats[c]["regime_diff"] <= 1e-4 * stats[c]["softened"], stats
    assert e_mix[50] < 2e-5, stats
    # the mixed error grows no faster than the problem amplifies an FP64
    # perturbation (with a factor 2 of margin)
    assert e_mix[100] / e_mix[50] <= 2.0 * e_per[100] / e_per[50], stats
