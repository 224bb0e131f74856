"""CUDA step vs the oracle: the parity tests proper (GPU).

Bars (written in each test):

* plain and fused FP64 paths: bit-identical to the oracle (u, ud, udd,
  force, body_force, damage, nlist, n_neigh), which itself reproduces the
  reference goldens;
* mixed path: max|u - u_oracle| / max|u_oracle| < 1e-5 and the broken-bond
  mask identical to the oracle's.
"""
import ctypes

import numpy as np
import pytest

from oracle import cl_step
from tests import known_answers
from tests.conftest import cuda_available
from tests.gpu_helpers import (breaking_setup, lattice, pull_bcs, rel_err,
                               run_integrator, run_oracle)
from tests.plate_setup import (BOND_STIFFNESS, CRITICAL_STRETCH, DISP_MAGS,
                               DT, STEPS)

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(),
                                 reason="needs a CUDA GPU")]

MIXED_TOL = 1e-5


@pytest.fixture(scope="module")
def torch():
    import torch as _torch
    return _torch


@pytest.fixture(scope="module")
def L():
    from probabilistic_peridynamics_gb300 import _lib
    return _lib.lib()


def _dev(torch, a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=dtype)).cuda()


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


# ----------------------------------------------------------- known answers
@pytest.mark.parametrize("name", list(known_answers.bond_force_cases()))
def test_known_answer_bond_force(torch, L, name):
    from probabilistic_peridynamics_gb300 import _lib
    case = known_answers.bond_force_cases()[name]
    n = case["r0"].shape[0]
    mn = case["nlist"].shape[1]
    d = dict(u=_dev(torch, case["u"], np.float64),
             r0=_dev(torch, case["r0"], np.float64),
             vols=_dev(torch, case["vols"], np.float64),
             nlist=_dev(torch, case["nlist"], np.int32),
             fct=_dev(torch, np.zeros((n, 3)), np.int32),
             fcv=_dev(torch, np.zeros((n, 3)), np.float64),
             force=torch.zeros((n, 3), dtype=torch.float64, device="cuda"),
             body=torch.zeros((n, 3), dtype=torch.float64, device="cuda"),
             sc=(None if case["sc"] is None
                 else _dev(torch, case["sc"], np.float64)))
    a = _lib.BondForceArgs()
    a.nnodes, a.max_neigh = n, mn
    a.u, a.force, a.body_force = _p(d["u"]), _p(d["force"]), _p(d["body"])
    a.r0, a.vols, a.nlist = _p(d["r0"]), _p(d["vols"]), _p(d["nlist"])
    a.fc_types, a.fc_values = _p(d["fct"]), _p(d["fcv"])
    a.stiffness_corrections = _p(d["sc"])
    a.bond_stiffness, a.critical_stretch, a.fc_scale = (
        case["k"], case["s0"], 1.0)
    assert L.pp_bond_force(ctypes.byref(a), None) == 0
    torch.cuda.synchronize()
    nl_ref = case["nlist"].copy()
    f_ref, _ = cl_step.bond_force(
        case["u"], case["r0"], case["vols"], nl_ref, np.zeros((n, 3)),
        np.zeros((n, 3)), 1.0, case["k"], case["s0"],
        stiffness_corrections=case["sc"])
    force = d["force"].cpu().numpy()
    assert np.array_equal(force, f_ref)  # bit-exact vs oracle
    assert np.array_equal(d["nlist"].cpu().numpy(), nl_ref)
    if case["force"] is not None:
        assert np.allclose(force, case["force"])
    if "nlist_out" in case:
        assert np.array_equal(d["nlist"].cpu().numpy(), case["nlist_out"])
        fam = _dev(torch, case["family"], np.int32)
        nn = torch.zeros(n, dtype=torch.int32, device="cuda")
        dmg = torch.zeros(n, dtype=torch.float64, device="cuda")
        assert L.pp_damage(_p(d["nlist"]), _p(fam), _p(nn), _p(dmg), n, mn,
                           None) == 0
        assert np.array_equal(nn.cpu().numpy(), case["n_neigh_out"])
        assert np.allclose(dmg.cpu().numpy(), case["damage_out"])


@pytest.mark.parametrize("idx", range(len(known_answers.update_cases())))
def test_known_answer_update(torch, L, idx):
    kind, inp, exp = known_answers.update_cases()[idx]
    u = _dev(torch, inp["u"], np.float64)
    f = _dev(torch, inp["force"], np.float64)
    bt = _dev(torch, inp["bc_types"], np.int32)
    bv = _dev(torch, inp["bc_values"], np.float64)
    if kind == "euler":
        assert L.pp_update_displacement_euler(
            _p(f), _p(u), _p(bt), _p(bv), inp["bc_scale"], inp["dt"], 3,
            None) == 0
        assert np.array_equal(u.cpu().numpy(), exp["u"])
        return
    ud = _dev(torch, inp["ud"], np.float64)
    udd = _dev(torch, inp["udd"], np.float64)
    rho = _dev(torch, inp["densities"], np.float64)
    fn = (L.pp_update_displacement_euler_cromer if kind == "euler_cromer"
          else L.pp_update_displacement_velocity_verlet)
    assert fn(_p(f), _p(u), _p(ud), _p(udd), _p(bt), _p(bv), _p(rho),
              inp["bc_scale"], inp["damping"], inp["dt"], 3, None) == 0
    assert np.array_equal(u.cpu().numpy(), exp["u"])
    assert np.array_equal(ud.cpu().numpy(), exp["ud"])
    assert np.array_equal(udd.cpu().numpy(), exp["udd"])


# ------------------------------------------------------------ plate goldens
_KINDS = {"euler": "EulerCUDA", "euler_cromer": "EulerCromerCUDA",
          "velocity_verlet": "VelocityVerletCUDA"}
_PREFIX = {"euler": "euler", "euler_cromer": "ec", "velocity_verlet": "vv"}


def _make(kind, **kw):
    import probabilistic_peridynamics_gb300 as pp
    cls = getattr(pp, _KINDS[kind])
    if kind == "euler":
        return cls(dt=DT, **kw)
    return cls(dt=DT, damping=0.0, **kw)


def _plate_setup(plate, kind):
    s = dict(plate)
    s["k"], s["s0"], s["dt"] = BOND_STIFFNESS, CRITICAL_STRETCH, DT
    if kind == "euler":
        s["densities"] = None
    return s


@pytest.mark.parametrize("kind", list(_KINDS))
@pytest.mark.parametrize("mode", ["plain", "fused64", "fused64_run",
                                  "mixed", "mixed_run"])
def test_plate_goldens(plate, golden, kind, mode):
    setup = _plate_setup(plate, kind)
    fused = mode != "plain"
    precision = "mixed" if mode.startswith("mixed") else "float64"
    integ = _make(kind, fused=fused, precision=precision)
    out = run_integrator(integ, setup, STEPS, DISP_MAGS,
                         use_run=mode.endswith("_run"))
    ref = run_oracle(kind, setup, STEPS, DISP_MAGS)
    u, ud, udd, force, body, damage, nlist, n_neigh = out
    pre = _PREFIX[kind]
    assert np.array_equal(nlist, ref[6])
    assert np.array_equal(n_neigh, ref[7])
    assert np.array_equal(nlist, golden[f"{pre}_nlist"])
    assert np.array_equal(damage, ref[5])
    if precision == "float64":
        for got, want in zip(out[:5], ref[:5]):
            assert np.array_equal(got, want)
        assert np.allclose(u, golden[f"{pre}_u"])
        assert np.allclose(force, golden[f"{pre}_force"])
    else:
        assert rel_err(u, ref[0]) < MIXED_TOL
        assert rel_err(force, ref[3]) < 1e-4
        if kind != "euler":
            assert rel_err(ud, ref[1]) < MIXED_TOL


# ------------------------------------------------ breaking 3-D lattice
@pytest.mark.parametrize("kind", list(_KINDS))
@pytest.mark.parametrize("mode", ["plain", "fused64", "mixed"])
def test_breaking_lattice(kind, mode):
    """Load-induced breaking on a 320-node lattice, 60 steps."""
    import probabilistic_peridynamics_gb300 as pp
    setup = breaking_setup(kind)
    steps = 60
    mags = 3e-3 * np.arange(1, steps + 1)
    cls = getattr(pp, _KINDS[kind])
    kw = dict(fused=mode != "plain",
              precision="mixed" if mode == "mixed" else "float64")
    integ = (cls(dt=setup["dt"], **kw) if kind == "euler"
             else cls(damping=0.5, dt=setup["dt"], **kw))
    out = run_integrator(integ, setup, steps, mags)
    ref = run_oracle(kind, setup, steps, mags,
                     damping=0.0 if kind == "euler" else 0.5)
    broken = int((setup["nlist"] != -1).sum() - (ref[6] != -1).sum())
    assert broken > 0  # the case exercises load-induced breaking
    if mode == "mixed":
        flips = int((out[6] != ref[6]).sum())
        assert flips == 0
        assert rel_err(out[0], ref[0]) < MIXED_TOL
    else:
        for got, want in zip(out, ref):
            assert np.array_equal(got, want)


# ---------------------------------------- n-linear, bond types, corrections
def _nlinear_setup(kind, corrections):
    from probabilistic_peridynamics_gb300.model import Model
    setup = breaking_setup(kind, 10, 6, 4)
    coords, nlist = setup["coords"], setup["nlist"]
    n, mn = nlist.shape
    mid = coords[:, 0].max() / 2
    left = coords[:, 0] < mid
    valid = nlist != -1
    jj = np.where(valid, nlist, 0)
    bt = np.where(left[:, None] & left[jj], 0,
                  np.where(~left[:, None] & ~left[jj], 1, 2))
    setup["bond_types"] = np.where(valid, bt, 0).astype(np.intc)
    k0 = 0.01
    ks = np.array([[k0, k0 / 2, -k0 / 4], [2 * k0, k0, -k0 / 2],
                   [1.5 * k0, 0.0, -k0 / 3]])
    ss = np.array([[0.010, 0.016, 0.024], [0.008, 0.014, 0.022],
                   [0.009, 0.015, 0.023]])
    k_tab, s_tab, c_tab, nbt, nreg = Model._set_damage_model(None, ks, ss)
    if corrections:
        rng = np.random.default_rng(7)
        sc = rng.uniform(0.9, 1.1, size=(n, mn))
        setup["stiffness_corrections"] = np.where(valid, sc, 0.0)
    return setup, k_tab, s_tab, c_tab, int(nbt), int(nreg)


@pytest.mark.parametrize("kind", list(_KINDS))
@pytest.mark.parametrize("mode", ["plain", "fused64", "mixed"])
@pytest.mark.parametrize("corrections", [False, True])
def test_nlinear_regimes(kind, mode, corrections):
    import probabilistic_peridynamics_gb300 as pp
    setup, k_tab, s_tab, c_tab, nbt, nreg = _nlinear_setup(kind,
                                                           corrections)
    steps = 50
    mags = 3e-3 * np.arange(1, steps + 1)
    cls = getattr(pp, _KINDS[kind])
    kw = dict(fused=mode != "plain",
              precision="mixed" if mode == "mixed" else "float64")
    integ = (cls(dt=setup["dt"], **kw) if kind == "euler"
             else cls(damping=0.5, dt=setup["dt"], **kw))
    out = run_integrator(integ, setup, steps, mags, bond_stiffness=k_tab,
                         critical_stretch=s_tab, plus_cs=c_tab,
                         nregimes=nreg, nbond_types=nbt)
    ref = run_oracle(kind, setup, steps, mags,
                     damping=0.0 if kind == "euler" else 0.5,
                     bond_stiffness=k_tab, critical_stretch=s_tab,
                     plus_cs=c_tab, nregimes=nreg)
    assert int((setup["nlist"] != -1).sum() - (ref[6] != -1).sum()) > 0
    if mode == "mixed":
        assert int((out[6] != ref[6]).sum()) == 0
        assert rel_err(out[0], ref[0]) < MIXED_TOL
    else:
        for got, want in zip(out, ref):
            assert np.array_equal(got, want)


def test_regimes_state_matches_oracle():
    """The regimes array itself (bond_force3, peridynamics.cl:345-360)."""
    import probabilistic_peridynamics_gb300 as pp
    setup, k_tab, s_tab, c_tab, nbt, nreg = _nlinear_setup("euler", False)
    steps = 40
    mags = 3e-3 * np.arange(1, steps + 1)
    integ = pp.EulerCUDA(dt=setup["dt"])
    run_integrator(integ, setup, steps, mags, bond_stiffness=k_tab,
                   critical_stretch=s_tab, plus_cs=c_tab, nregimes=nreg,
                   nbond_types=nbt)
    st = cl_step.Stepper(
        "euler", setup["dt"], setup["coords"], setup["volume"],
        setup["family"], setup["nlist"], setup["bc_types"],
        setup["bc_values"], setup["force_bc_types"],
        setup["force_bc_values"], k_tab, s_tab,
        bond_types=setup["bond_types"], plus_cs=c_tab, nregimes=nreg)
    for k in range(steps):
        st.step(mags[k], 0.0)
    regimes = integ.regimes_d.cpu().numpy()
    assert np.array_equal(regimes, st.regimes)
    assert np.any(st.regimes[st.nlist != -1] > 0)


# --------------------------------------------------------- Model.simulate
def test_model_simulate_plate(golden, tmp_path):
    """Model(...).simulate(...) end to end (test_regression.py:10-148)."""
    import probabilistic_peridynamics_gb300 as pp
    from probabilistic_peridynamics_gb300.mesh import write_vtk
    from tests.plate_setup import is_crack, is_displacement_boundary
    mesh = tmp_path / "plate.vtk"
    write_vtk(mesh, golden["points"], [("triangle", golden["cells_triangle"]),
                                       ("line", golden["cells_line"])])
    model = pp.Model(mesh, integrator=pp.EulerCUDA(dt=DT), horizon=0.1,
                     critical_stretch=CRITICAL_STRETCH,
                     bond_stiffness=BOND_STIFFNESS,
                     initial_crack=pp.initial_crack_helper(is_crack),
                     is_displacement_boundary=is_displacement_boundary)
    assert np.allclose(model.volume, golden["volume"])
    u, damage, (nlist, n_neigh), force, ud, data = model.simulate(
        steps=STEPS, displacement_bc_magnitudes=DISP_MAGS)
    assert np.allclose(u, golden["euler_u"])
    assert np.allclose(force, golden["euler_force"])
    assert np.allclose(damage, golden["euler_damage"])
    assert np.array_equal(np.sort(n_neigh), np.sort(golden["euler_n_neigh"]))
    # stateless: a second simulate gives identical results
    u2, damage2, conn2, force2, ud2, _ = model.simulate(
        steps=STEPS, displacement_bc_magnitudes=DISP_MAGS)
    assert np.array_equal(u, u2) and np.array_equal(force, force2)
    assert np.array_equal(nlist, conn2[0])


def test_model_restart():
    """Two 1-step simulates equal one 2-step simulate (test_model.py:1628)."""
    import probabilistic_peridynamics_gb300 as pp
    setup = breaking_setup("euler")
    mags = np.linspace(0, 0.00001 * 99 / 2, 100)
    for fused in (False, True):
        model = _lattice_model(pp.EulerCUDA(dt=setup["dt"], fused=fused),
                               setup)
        u, damage, conn, force, ud, _ = model.simulate(
            steps=1, displacement_bc_magnitudes=mags)
        u, damage, conn, force, ud, _ = model.simulate(
            steps=1, displacement_bc_magnitudes=mags, u=u, connectivity=conn,
            first_step=2)
        eu, edamage, econn, eforce, eud, _ = model.simulate(
            steps=2, displacement_bc_magnitudes=mags)
        assert np.array_equal(u, eu)
        assert np.array_equal(force, eforce)
        assert np.array_equal(conn[0], econn[0])


def _lattice_model(integ, setup, tmp=None):
    import tempfile
    import probabilistic_peridynamics_gb300 as pp
    from probabilistic_peridynamics_gb300.mesh import write_vtk
    d = tempfile.mkdtemp()
    mesh = f"{d}/lattice.vtk"
    write_vtk(mesh, setup["coords"], [])
    bc_t, bc_v = setup["bc_types"], setup["bc_values"]

    def is_bnd(x):
        i = int(np.argmin(np.sum((setup["coords"] - x) ** 2, axis=1)))
        return [float(bc_v[i, d]) if bc_t[i, d] else None for d in range(3)]

    return pp.Model(mesh, integrator=integ, horizon=3.015,
                    critical_stretch=setup["s0"], bond_stiffness=setup["k"],
                    transfinite=1, volume_total=float(setup["volume"].sum()),
                    dimensions=3, is_displacement_boundary=is_bnd)


def test_fused_run_graph_matches_steps():
    """pp_fused_run (graph replay) == step-by-step calls, bit for bit."""
    import probabilistic_peridynamics_gb300 as pp
    setup = breaking_setup("velocity_verlet")
    steps = 70
    mags = 3e-3 * np.arange(1, steps + 1)
    for precision in ("float64", "mixed"):
        outs = []
        for use_run in (False, True):
            integ = pp.VelocityVerletCUDA(damping=0.5, dt=setup["dt"],
                                          precision=precision)
            outs.append(run_integrator(integ, setup, steps, mags,
                                       use_run=use_run))
        for a, b in zip(*outs):
            assert np.array_equal(a, b)


# ------------------------------------------------------ every row width
@pytest.mark.parametrize("factor,width", [(1.0, 8), (2.0, 32), (2.3, 64),
                                          (3.015, 128), (3.5, 256)])
@pytest.mark.parametrize("mode", ["fused64", "mixed"])
def test_row_widths(factor, width, mode):
    """Rows of 8 to 256 slots: both bond-phase layouts of the mixed kernel
    (one warp per node up to 32 slots, four nodes per warp beyond) and the
    FP64 kernel's slot loops, with load-induced breaking."""
    import probabilistic_peridynamics_gb300 as pp
    coords, volume, horizon, family, nlist, n_neigh = lattice(9, 8, 8, 1.0,
                                                              factor)
    assert nlist.shape[1] == width
    bc_types, bc_values = pull_bcs(coords, 0)
    n = coords.shape[0]
    setup = dict(coords=coords, volume=volume, family=family, nlist=nlist,
                 n_neigh=n_neigh, bc_types=bc_types, bc_values=bc_values,
                 force_bc_types=np.zeros((n, 3), dtype=np.intc),
                 force_bc_values=np.zeros((n, 3)), nnodes=n, max_neigh=width,
                 k=0.01 * 122.0 / max(int(family.max()), 1), s0=0.02, dt=0.5)
    steps = 40
    mags = 4e-3 * np.arange(1, steps + 1)
    integ = pp.EulerCUDA(dt=setup["dt"], fused=True,
                         precision="mixed" if mode == "mixed" else "float64")
    out = run_integrator(integ, setup, steps, mags)
    ref = run_oracle("euler", setup, steps, mags)
    assert int((nlist != -1).sum() - (ref[6] != -1).sum()) > 0
    if mode == "mixed":
        assert int((out[6] != ref[6]).sum()) == 0
        assert np.array_equal(out[7], ref[7])
        assert rel_err(out[0], ref[0]) < MIXED_TOL
    else:
        for got, want in zip(out, ref):
            assert np.array_equal(got, want)


# ------------------------------------------------- force boundary conditions
@pytest.mark.parametrize("kind", list(_KINDS))
@pytest.mark.parametrize("mode", ["plain", "fused64", "mixed", "mixed_run",
                                  "mixed_untiled"])
def test_force_boundary_conditions(kind, mode):
    """A force on the x-max face (F / vol / n_face per node, as
    ``_set_boundary_conditions`` spreads it, ``peripy/model.py:1194-1209``)
    ramped over the steps, the x-min face clamped; bonds break under it.
    The mixed step on both layouts (tiled: the node update runs in the bond
    phase's lanes; untiled: in the node phase)."""
    import probabilistic_peridynamics_gb300 as pp
    setup = breaking_setup(kind)
    coords, vol = setup["coords"], setup["volume"]
    n = coords.shape[0]
    right = coords[:, 0] >= coords[:, 0].max() - 1e-9
    left = coords[:, 0] <= coords[:, 0].min() + 1e-9
    bc_types = np.zeros((n, 3), dtype=np.intc)
    bc_types[left] = 1
    setup["bc_types"], setup["bc_values"] = bc_types, np.zeros((n, 3))
    fct = np.zeros((n, 3), dtype=np.intc)
    fcv = np.zeros((n, 3))
    fct[right, 0] = 1
    fcv[right, 0] = 1.0 / vol[right] / right.sum()
    setup["force_bc_types"], setup["force_bc_values"] = fct, fcv
    steps = 60
    dmags = np.zeros(steps)
    fmags = 0.02 * np.arange(1, steps + 1)
    cls = getattr(pp, _KINDS[kind])
    kw = dict(fused=mode != "plain",
              precision="mixed" if mode.startswith("mixed") else "float64")
    if mode.startswith("mixed"):
        kw.update(tiled=mode != "mixed_untiled", autotune=False)
    integ = (cls(dt=setup["dt"], **kw) if kind == "euler"
             else cls(damping=0.5, dt=setup["dt"], **kw))
    out = run_integrator(integ, setup, steps, dmags, force_mags=fmags,
                         use_run=mode.endswith("_run"))
    if mode.startswith("mixed"):
        assert (integ.tiling is not None) == (mode != "mixed_untiled")
    ref = run_oracle(kind, setup, steps, dmags, force_mags=fmags,
                     damping=0.0 if kind == "euler" else 0.5)
    assert int((setup["nlist"] != -1).sum() - (ref[6] != -1).sum()) > 0
    assert np.any(ref[4][right, 0] != 0.0)  # the force reached the face
    if mode.startswith("mixed"):
        assert int((out[6] != ref[6]).sum()) == 0
        assert rel_err(out[0], ref[0]) < MIXED_TOL
        assert rel_err(out[4], ref[4]) < MIXED_TOL
    else:
        for got, want in zip(out, ref):
            assert np.array_equal(got, want)


@pytest.mark.parametrize("kind", ["euler", "euler_cromer", "velocity_verlet"])
@pytest.mark.parametrize("mode", ["plain", "fused64", "mixed"])
def test_nonuniform_volumes_and_densities(kind, mode):
    """Node volumes (bond weights k*vol_j) and densities that differ per
    node and per component, with breaking."""
    import probabilistic_peridynamics_gb300 as pp
    setup = breaking_setup(kind)
    n = setup["nnodes"]
    rng = np.random.default_rng(11)
    setup["volume"] = rng.uniform(0.7, 1.3, n)
    if kind != "euler":
        setup["densities"] = rng.uniform(30.0, 70.0, (n, 3))
    steps = 60
    mags = 3e-3 * np.arange(1, steps + 1)
    cls = getattr(pp, _KINDS[kind])
    kw = dict(fused=mode != "plain",
              precision="mixed" if mode == "mixed" else "float64")
    integ = (cls(dt=setup["dt"], **kw) if kind == "euler"
             else cls(damping=0.5, dt=setup["dt"], **kw))
    out = run_integrator(integ, setup, steps, mags)
    ref = run_oracle(kind, setup, steps, mags,
                     damping=0.0 if kind == "euler" else 0.5)
    assert int((setup["nlist"] != -1).sum() - (ref[6] != -1).sum()) > 0
    if mode == "mixed":
        assert int((out[6] != ref[6]).sum()) == 0
        assert rel_err(out[0], ref[0]) < MIXED_TOL
        if kind != "euler":
            assert rel_err(out[1], ref[1]) < MIXED_TOL
    else:
        for got, want in zip(out, ref):
            assert np.array_equal(got, want)
