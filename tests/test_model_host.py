"""``Model``'s host-side logic without a GPU (``peripy/model.py:42-1575``).

A recording integrator (an :class:`Integrator` that keeps what ``Model``
hands it and does no device work, with ``context`` None like PeriPy's CPU
integrator) lets the constructor and ``simulate`` run on the host: argument
checks and their exceptions, mesh reading and node volumes, the compact
neighbour-list layout and the initial crack (against the reference's golden
connectivity), the damage-model tables (the ``plus_cs`` recurrence),
boundary conditions, force boundary values, tips, densities and bond types,
and the sequence of integrator calls ``simulate`` makes.
"""
import numpy as np
import pytest

from probabilistic_peridynamics_gb300.integrators import Integrator


class HostIntegrator(Integrator):
    """Records the calls Model makes; no device work."""

    def __init__(self, dt=1.0):
        self.dt = dt
        self.context = None
        self.calls = []

    def __call__(self, displacement_bc_magnitude, force_bc_magnitude):
        self.calls.append((displacement_bc_magnitude, force_bc_magnitude))

    def build(self, *args):
        self.built = args

    def create_buffers(self, *args):
        self.buffers = args
        self.state = list(args[5:11])  # u, ud, udd, force, body_force, damage

    def write(self, u, ud, udd, force, body_force, damage, nlist, n_neigh):
        self.writes = getattr(self, "writes", 0) + 1
        return u, ud, udd, force, body_force, damage, nlist, n_neigh

    def _build_special(self):
        pass

    def _create_special_buffers(self):
        pass


@pytest.fixture(scope="module")
def mesh(golden, tmp_path_factory):
    from probabilistic_peridynamics_gb300.mesh import write_vtk
    path = tmp_path_factory.mktemp("mesh") / "plate.vtk"
    write_vtk(path, golden["points"], [("triangle", golden["cells_triangle"]),
                                       ("line", golden["cells_line"])])
    return path


def _model(mesh, **kw):
    import probabilistic_peridynamics_gb300 as pp
    args = dict(integrator=HostIntegrator(), horizon=0.1,
                critical_stretch=0.005, bond_stiffness=1.0)
    args.update(kw)
    return pp.Model(mesh, **args)


def test_integrator_and_dimension_checks(mesh):
    import probabilistic_peridynamics_gb300 as pp
    with pytest.raises(pp.InvalidIntegrator):
        pp.Model(mesh, integrator=object(), horizon=0.1,
                 critical_stretch=0.005, bond_stiffness=1.0)
    with pytest.raises(pp.DimensionalityError):
        _model(mesh, dimensions=4)
    m = _model(mesh)
    assert m.mesh_elements.connectivity == "triangle"
    assert m.mesh_elements.boundary == "line"


def test_mesh_and_volume(mesh, golden):
    m = _model(mesh)
    assert np.array_equal(m.coords, golden["points"])
    assert np.array_equal(m.mesh_connectivity, golden["cells_triangle"])
    assert np.array_equal(m.mesh_boundary, golden["cells_line"])
    assert np.allclose(m.volume, golden["volume"])
    n = golden["points"].shape[0]
    assert m.nnodes == n and m.degrees_freedom == 3
    # volume given as an argument is taken as it is (with a warning)
    vol = np.full(n, 0.5)
    with pytest.warns(UserWarning):
        m2 = _model(mesh, volume=vol)
    assert np.array_equal(m2.volume, vol)
    with pytest.raises(ValueError):
        _model(mesh, volume=np.ones(n + 1))
    with pytest.raises(TypeError):
        _model(mesh, volume=[1.0] * n)


def test_compact_layout_and_crack(mesh, golden):
    """Without a device context the rows are compact (width family.max())
    and 0-padded; the sets equal the reference's KD-tree rows, and the crack
    leaves the golden counts."""
    import probabilistic_peridynamics_gb300 as pp
    from tests.plate_setup import is_crack
    m = _model(mesh)
    nlist, n_neigh = m.initial_connectivity
    assert np.array_equal(m.family, golden["cy_n_neigh_basic"])
    assert nlist.shape[1] == int(m.family.max()) == m.max_neighbours
    ref = golden["cy_nlist_basic"]
    for i in range(nlist.shape[0]):
        k = n_neigh[i]
        assert np.array_equal(np.sort(nlist[i, :k]), np.sort(ref[i, :k]))
        assert np.all(nlist[i, k:] == 0)
    mc = _model(mesh, initial_crack=pp.initial_crack_helper(is_crack))
    _, n_crack = mc.initial_connectivity
    assert np.array_equal(n_crack, golden["cy_n_neigh_crack"])
    assert np.array_equal(mc.family, m.family)


def _plus_cs(k, s):
    """plus_cs[r] = plus_cs[r-1] + k[r-1] s[r-1] - k[r] s[r-1] (the force
    is continuous across regimes), for one bond type or a table of them."""
    k = np.atleast_2d(np.asarray(k, dtype=np.float64))
    s = np.atleast_2d(np.asarray(s, dtype=np.float64))
    c = np.zeros_like(k)
    for r in range(1, k.shape[1]):
        c[:, r] = (c[:, r - 1] + k[:, r - 1] * s[:, r - 1]
                   - k[:, r] * s[:, r - 1])
    return c


@pytest.mark.parametrize("kind", ["list", "array"])
def test_damage_model_tables(mesh, kind):
    k1, s1 = [1.0, 0.5, 0.25], [0.001, 0.002, 0.003]
    k2 = [[1.0, 0.5], [2.0, 1.0], [3.0, 0.1]]
    s2 = [[0.001, 0.002], [0.003, 0.004], [0.001, 0.005]]
    wrap = (lambda x: x) if kind == "list" else np.array
    m = _model(mesh, bond_stiffness=wrap(k1), critical_stretch=wrap(s1))
    assert (m.nregimes, m.nbond_types) == (3, 1)
    assert np.array_equal(m.plus_cs, _plus_cs(k1, s1)[0])

    def bond_type(x, y):
        return 0 if x[0] < 0.5 and y[0] < 0.5 else (
            1 if x[0] >= 0.5 and y[0] >= 0.5 else 2)
    m = _model(mesh, bond_stiffness=wrap(k2), critical_stretch=wrap(s2),
               is_bond_type=bond_type)
    assert (m.nregimes, m.nbond_types) == (2, 3)
    assert np.array_equal(m.plus_cs, _plus_cs(k2, s2))
    assert set(np.unique(m.bond_types)) <= {0, 1, 2}


def test_damage_model_errors(mesh):
    import probabilistic_peridynamics_gb300 as pp
    with pytest.raises(pp.DamageModelError):
        _model(mesh, bond_stiffness=[1.0, 0.5], critical_stretch=[0.002,
                                                                  0.001])
    with pytest.raises(TypeError):
        _model(mesh, bond_stiffness=[1.0, 0.5], critical_stretch=0.005)
    with pytest.raises(ValueError):
        _model(mesh, bond_stiffness=[1.0, 0.5],
               critical_stretch=[0.001, 0.002, 0.003])
    with pytest.raises(ValueError):
        _model(mesh, bond_stiffness=1.0, critical_stretch=-0.005)
    with pytest.raises(TypeError):
        _model(mesh, bond_stiffness=1, critical_stretch=1)


def test_bond_type_function_checks(mesh):
    k2, s2 = [[1.0], [2.0]], [[0.001], [0.002]]
    with pytest.raises(TypeError):
        _model(mesh, bond_stiffness=k2, critical_stretch=s2, is_bond_type=1)
    with pytest.raises(TypeError):
        _model(mesh, bond_stiffness=k2, critical_stretch=s2,
               is_bond_type=lambda x, y: 0.5)
    with pytest.raises(ValueError):
        _model(mesh, bond_stiffness=k2, critical_stretch=s2,
               is_bond_type=lambda x, y: 2)
    with pytest.raises(ValueError):
        _model(mesh, bond_stiffness=k2, critical_stretch=s2,
               is_bond_type=lambda x, y: -1)


def test_boundary_conditions_and_tips(mesh, golden):
    def bnd(x):
        return [-1.0, 0.0, None] if x[0] < 0.1 else [None, None, None]

    def fbnd(x):
        return [None, None, 2.0] if x[0] > 0.9 else [None, None, None]

    def tip(x):
        if x[0] > 0.95:
            return [None, "right", ("right", "far")]
        return [None, None, None]
    m = _model(mesh, is_displacement_boundary=bnd, is_force_boundary=fbnd,
               is_tip=tip)
    x = m.coords[:, 0]
    left, right = x < 0.1, x > 0.9
    assert np.all(m.bc_types[left, :2] == 1)
    assert np.all(m.bc_types[left, 2] == 0)
    assert np.all(m.bc_values[left, 0] == -1.0)
    assert np.all(m.bc_types[~left] == 0)
    # force boundary values: F / volume[i], spread over the force nodes
    nforce = int(right.sum())
    assert np.allclose(m.force_bc_values[right, 2],
                       2.0 / m.volume[right] / nforce)
    assert np.all(m.force_bc_types[right, 2] == 1)
    far = x > 0.95
    assert m.ntips["right"] == 2 * int(far.sum())
    assert m.ntips["far"] == int(far.sum())
    assert all(j == 1 for i, j in m.tip_types["right"][::2])
    assert m.ntips["model"] == m.nnodes
    with pytest.raises(TypeError):
        _model(mesh, is_displacement_boundary=lambda x: [None, None])
    with pytest.raises(TypeError):
        _model(mesh, is_tip=lambda x: None)


def test_densities(mesh):
    n = _model(mesh).nnodes
    m = _model(mesh, is_density=lambda x: 2.0)
    assert m.densities.shape == (n, 3) and np.all(m.densities == 2.0)
    with pytest.raises(TypeError):
        _model(mesh, is_density=lambda x: 2)
    with pytest.raises(TypeError):
        _model(mesh, is_density=2.0)
    with pytest.warns(UserWarning):
        m = _model(mesh, density=np.full(n, 3.0))
    assert np.all(m.densities == 3.0)
    with pytest.raises(ValueError):
        _model(mesh, density=np.ones(n + 2))


def test_simulate_calls(mesh, tmp_path):
    """One integrator call per step with that step's magnitudes, a write at
    every write step plus the final one, and the recorded steps."""
    m = _model(mesh)
    integ = m.integrator
    mags = np.linspace(1e-6, 1e-5, 10)
    fmags = np.linspace(0.0, 1.0, 10)
    u, damage, (nlist, n_neigh), force, ud, data = m.simulate(
        steps=10, displacement_bc_magnitudes=mags,
        force_bc_magnitudes=fmags, write=4, write_path=tmp_path)
    assert integ.calls == list(zip(mags, fmags))
    assert integ.writes == 2 + 1
    assert list(data["model"]["step"]) == [4, 8]
    assert (tmp_path / "U_4.vtk").exists() and (tmp_path / "U_8.vtk").exists()
    # restart: first_step carries on the magnitudes and write numbering
    integ.calls.clear()
    m.simulate(steps=3, displacement_bc_magnitudes=mags,
               force_bc_magnitudes=fmags, first_step=5)
    assert integ.calls == list(zip(mags[4:7], fmags[4:7]))


def test_simulate_argument_checks(mesh):
    m = _model(mesh)
    n, w = m.nnodes, m.max_neighbours
    with pytest.raises(ValueError):
        m.simulate(steps=5, displacement_bc_magnitudes=np.zeros(3))
    with pytest.raises(TypeError):
        m.simulate(steps=2, displacement_bc_magnitudes=[0.0, 0.0])
    with pytest.raises(ValueError):
        m.simulate(steps=5, force_bc_magnitudes=np.zeros(4))
    with pytest.raises(TypeError):
        m.simulate(steps=2, force_bc_magnitudes=(0.0, 0.0))
    nl, nn = m.initial_connectivity
    with pytest.raises(ValueError):
        m.simulate(steps=1, connectivity=(nl, nn, nn))
    with pytest.raises(TypeError):
        m.simulate(steps=1, connectivity=[nl, nn])
    with pytest.raises(ValueError):
        m.simulate(steps=1, regimes=np.zeros((n, w + 1), dtype=np.intc))
    with pytest.raises(TypeError):
        m.simulate(steps=1, regimes=[[0] * w] * n)
    # a new damage model may not change the number of bond types
    with pytest.raises(ValueError):
        m.simulate(steps=1, bond_stiffness=[[1.0], [2.0]],
                   critical_stretch=[[0.001], [0.002]])
    # the initial connectivity is left as it is: simulate works on copies
    before = nl.copy()
    m.simulate(steps=2)
    assert np.array_equal(m.initial_connectivity[0], before)
    assert m.integrator.buffers[0] is not m.initial_connectivity[0]


def test_write_mesh_and_cached_arrays(mesh, golden, tmp_path):
    """write_mesh (model.py:505-534) writes the nodes, the cells and the
    point data; with write_path the set-up arrays are cached as files."""
    from probabilistic_peridynamics_gb300.mesh import read_vtk
    from probabilistic_peridynamics_gb300.model import read_array
    cache = tmp_path / "cache"
    m = _model(mesh, write_path=cache, is_density=lambda x: 2.0)
    for name in ("volume", "family", "nlist", "n_neigh", "density"):
        assert read_array(cache, name) is not None
    assert np.array_equal(read_array(cache, "volume"), m.volume)
    assert np.array_equal(read_array(cache, "nlist"),
                          m.initial_connectivity[0])
    out = tmp_path / "state.vtk"
    damage = np.linspace(0.0, 1.0, m.nnodes)
    u = np.arange(3 * m.nnodes, dtype=np.float64).reshape(-1, 3)
    m.write_mesh(out, damage, u)
    back = read_vtk(out)
    assert np.array_equal(back.points, m.coords)
    assert np.array_equal(back.cells_dict["triangle"],
                          golden["cells_triangle"])
    assert np.array_equal(back.cells_dict["line"], golden["cells_line"])
    # the point data follow the cells: damage then displacements
    raw = out.read_bytes()
    assert b"POINT_DATA %d" % m.nnodes in raw
    assert b"damage 1 %d double" % m.nnodes in raw
    assert b"displacements 3 %d double" % m.nnodes in raw
    at = raw.index(b"damage 1 %d double\n" % m.nnodes) + len(
        b"damage 1 %d double\n" % m.nnodes)
    got = np.frombuffer(raw[at:at + 8 * m.nnodes], dtype=">f8")
    assert np.array_equal(got, damage)
