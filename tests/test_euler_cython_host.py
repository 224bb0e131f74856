"""The GPU ``Euler`` (PeriPy's CPU integrator on the device): the parts
that need no GPU -- its drop-in surface and argument checks, mirrored
from ``peripy/integrators.py:303-459``, and the host-side validation of
the ``pp_cy_*`` entry points."""
import numpy as np
import pytest


def test_surface():
    import probabilistic_peridynamics_gb300 as pp
    e = pp.Euler(dt=1e-3)
    assert e.context is None  # Model then builds the compact layout
    assert isinstance(e, pp.Integrator)
    assert e._build_special() is None
    assert e._create_special_buffers() is None
    with pytest.raises(TypeError):
        pp.Euler(1e-3, device_context=object())


@pytest.mark.parametrize("which", ["bond_types", "stiffness_corrections",
                                   "densities"])
def test_build_rejects_what_the_reference_rejects(which):
    import probabilistic_peridynamics_gb300 as pp
    e = pp.Euler(dt=1e-3)
    n = 4
    extra = dict(stiffness_corrections=None, bond_types=None, densities=None)
    extra[which] = np.ones((n, 3))
    with pytest.raises(ValueError, match=which):
        e.build(n, 3, 2, np.zeros((n, 3)), np.ones(n), np.ones(n, np.intc),
                np.zeros((n, 3), np.intc), np.zeros((n, 3)),
                np.zeros((n, 3), np.intc), np.zeros((n, 3)),
                extra["stiffness_corrections"], extra["bond_types"],
                extra["densities"])


def test_create_buffers_rejects_nlinear_and_types():
    import probabilistic_peridynamics_gb300 as pp
    e = pp.Euler(dt=1e-3)
    z = np.zeros((2, 3))
    with pytest.raises(ValueError, match="n-linear"):
        e.create_buffers(None, None, 1.0, 0.01, None, z, z, z, z, z, None,
                         None, 2, 1)
    with pytest.raises(ValueError, match="n-material"):
        e.create_buffers(None, None, 1.0, 0.01, None, z, z, z, z, z, None,
                         None, 1, 2)


def test_entry_point_validation_without_gpu():
    from probabilistic_peridynamics_gb300 import _lib
    L = _lib.lib()
    inv, wide = _lib.PP_ERROR_INVALID_VALUE, _lib.PP_ERROR_MAX_NEIGH
    assert L.pp_cy_break_bonds(None, None, None, None, 5, 2000, 0.1,
                               None) == wide
    assert L.pp_cy_break_bonds(None, None, None, None, 5, 4, 0.1,
                               None) == inv
    assert L.pp_cy_break_bonds(None, None, None, None, 0, 4, 0.1,
                               None) == _lib.PP_SUCCESS
    assert L.pp_cy_bond_force(None, None, None, None, None, 1.0, None, None,
                              0.0, 5, 2000, None, None) == wide
    assert L.pp_cy_bond_force(None, None, None, None, None, 1.0, None, None,
                              0.0, 5, 4, None, None) == inv
    assert L.pp_cy_break_and_force(None, None, None, None, None, 1.0, 0.1,
                                   None, None, 0.0, 5, 2000, None, None,
                                   None) == wide
    assert L.pp_cy_break_and_force(None, None, None, None, None, 1.0, 0.1,
                                   None, None, 0.0, 5, 4, None, None,
                                   None) == inv
    assert L.pp_cy_update_displacement(None, None, None, None, 0.0, 1.0, -1,
                                       None) == inv
    assert L.pp_cy_damage(None, None, 3, None, None) == inv
    assert L.pp_cy_damage(None, None, 0, None, None) == _lib.PP_SUCCESS
