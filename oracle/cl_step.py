"""NumPy restatement of PeriPy's OpenCL time step (TEST INFRASTRUCTURE).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may use this module, as the checker.  Nothing in the product package
imports it.

Every function follows one reference kernel, cited by file:line:

* :func:`bond_force`  -- ``peripy/cl/peridynamics.cl:4-565``
  (``bond_force1`` .. ``bond_force4``; the variant is chosen by which of
  ``stiffness_corrections`` / ``bond_types`` are given, exactly as
  ``peripy/integrators.py:109-148`` does).
* :func:`damage`      -- ``peripy/cl/peridynamics.cl:568-610``.
* :func:`update_euler`            -- ``peripy/cl/euler.cl:3-24``.
* :func:`update_euler_cromer`     -- ``peripy/cl/euler_cromer.cl:3-35``.
* :func:`update_velocity_verlet`  -- ``peripy/cl/velocity_verlet.cl:3-36``.

Arithmetic is IEEE binary64 with no fused multiply-add, evaluated in the
same association order as the OpenCL C expressions.  The per-node reduction
reproduces the work-group tree ``cache[l] += cache[l + i]`` for
``i = max_neigh/2 .. 1`` (``peridynamics.cl:107-115``), so results are
bit-reproducible for a given input, independent of the evaluation platform.
"""
import numpy as np


def tree_sum(a):
    """Sum ``a`` (n, L) over axis 1 in the work-group tree order.

    ``L`` must be a power of two (``peripy/model.py:575-578`` pads ``nlist``
    to the next power of two for device integrators).  Step ``i`` adds slot
    ``l + i`` into slot ``l`` for ``l < i`` (``peridynamics.cl:107-115``).
    """
    a = np.array(a, dtype=np.float64, copy=True)
    width = a.shape[1]
    if width & (width - 1):
        raise ValueError("max_neigh must be a power of two, got %d" % width)
    while width > 1:
        width //= 2
        a = a[:, :width] + a[:, width:2 * width]
    return a[:, 0]


def _bond_geometry(u, r0, nlist):
    """Stretch and deformed bond vector per slot (peridynamics.cl:65-75)."""
    nnodes = nlist.shape[0]
    valid = nlist != -1
    jj = np.where(valid, nlist, 0)
    ii = np.arange(nnodes)[:, None]
    xi_x = r0[jj, 0] - r0[ii, 0]
    xi_y = r0[jj, 1] - r0[ii, 1]
    xi_z = r0[jj, 2] - r0[ii, 2]
    xe_x = u[jj, 0] - u[ii, 0] + xi_x
    xe_y = u[jj, 1] - u[ii, 1] + xi_y
    xe_z = u[jj, 2] - u[ii, 2] + xi_z
    xi = np.sqrt(xi_x * xi_x + xi_y * xi_y + xi_z * xi_z)
    y = np.sqrt(xe_x * xe_x + xe_y * xe_y + xe_z * xe_z)
    s = (y - xi) / xi
    return valid, jj, s, y, (xe_x, xe_y, xe_z)


def bond_force(u, r0, vols, nlist, fc_types, fc_values, fc_scale,
               bond_stiffness, critical_stretch, stiffness_corrections=None,
               bond_types=None, regimes=None, plus_cs=None, nregimes=1):
    """One bond-force pass; mutates ``nlist`` (and ``regimes``) in place.

    Follows ``bond_force1`` (``peridynamics.cl:4-131``) when neither
    ``stiffness_corrections`` nor ``bond_types`` is given, ``bond_force2``
    (:134-262) with corrections only, ``bond_force3`` (:265-414) with bond
    types only and ``bond_force4`` (:417-565) with both.  For the n-linear
    variants ``bond_stiffness``, ``critical_stretch`` and ``plus_cs`` are the
    (nbond_types, nregimes) tables flattened row-major.

    :returns: ``(force, body_force)``, each (nnodes, 3) float64.
    """
    u = np.asarray(u, dtype=np.float64).reshape(-1, 3)
    r0 = np.asarray(r0, dtype=np.float64).reshape(-1, 3)
    vols = np.asarray(vols, dtype=np.float64)
    nnodes, width = nlist.shape
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        valid, jj, s, y, xe = _bond_geometry(u, r0, nlist)
        vol_j = vols[jj]
        if bond_types is None:
            k = np.float64(bond_stiffness)
            s0 = np.float64(critical_stretch)
            intact = valid & (s < s0)
            broken = valid & ~intact
            if stiffness_corrections is None:
                f = s * k * vol_j
            else:
                f = s * k * stiffness_corrections * vol_j
        else:
            nr = int(nregimes)
            k_tab = np.asarray(bond_stiffness, dtype=np.float64).ravel()
            s_tab = np.asarray(critical_stretch, dtype=np.float64).ravel()
            c_tab = np.asarray(plus_cs, dtype=np.float64).ravel()
            bt = bond_types.astype(np.int64)
            r = np.where(valid, regimes, 0).astype(np.int64)
            cur = s_tab[bt * nr + r]
            below = s < cur
            prev = s_tab[bt * nr + np.maximum(r - 1, 0)]
            dec = valid & below & (r > 0) & (s < prev)
            inc = valid & ~below
            r_new = r - dec + inc
            changed = dec | inc
            regimes[changed] = r_new[changed]
            broken = valid & (r_new >= nr)
            intact = valid & ~broken
            rc = np.minimum(r_new, nr - 1)
            k_sel = k_tab[bt * nr + rc]
            c_sel = c_tab[bt * nr + rc]
            if stiffness_corrections is None:
                f = (s * k_sel + c_sel) * vol_j
            else:
                f = (s * k_sel + c_sel) * stiffness_corrections * vol_j
        nlist[broken] = -1
        comps = []
        for comp in xe:
            c = comp / y
            comps.append(np.where(intact, f * c, 0.0))
    body_force = np.stack([tree_sum(c) for c in comps], axis=1)
    force = body_force.copy()
    fc_values = np.asarray(fc_values, dtype=np.float64).reshape(-1, 3)
    loaded = np.asarray(fc_types).reshape(-1, 3) != 0
    force[loaded] = body_force[loaded] + fc_scale * fc_values[loaded]
    return force, body_force


def damage(nlist, family):
    """Intact-bond count and damage (peridynamics.cl:568-610)."""
    count = tree_sum((nlist != -1).astype(np.float64))
    n_neigh = count.astype(np.intc)
    dmg = 1.0 - n_neigh.astype(np.float64) / np.asarray(
        family, dtype=np.float64)
    return n_neigh, dmg


def update_euler(force, u, bc_types, bc_values, bc_scale, dt):
    """In-place Euler update of ``u`` (euler.cl:21-23)."""
    f = force.reshape(-1)
    uf = u.reshape(-1)
    bt = np.asarray(bc_types).reshape(-1)
    bv = np.asarray(bc_values, dtype=np.float64).reshape(-1)
    uf[:] = np.where(bt == 0, uf + dt * f, bc_scale * bv)


def update_euler_cromer(force, u, ud, udd, bc_types, bc_values, densities,
                        bc_scale, damping, dt):
    """In-place Euler-Cromer update (euler_cromer.cl:53-58)."""
    f = force.reshape(-1)
    uf, udf, uddf = u.reshape(-1), ud.reshape(-1), udd.reshape(-1)
    bt = np.asarray(bc_types).reshape(-1)
    bv = np.asarray(bc_values, dtype=np.float64).reshape(-1)
    rho = np.asarray(densities, dtype=np.float64).reshape(-1)
    uddi = (f - damping * udf) / rho
    uddf[:] = uddi
    udf[:] = udf + uddi * dt
    uf[:] = np.where(bt == 0, uf + dt * udf, bc_scale * bv)


def update_velocity_verlet(force, u, ud, udd, bc_types, bc_values, densities,
                           bc_scale, damping, dt):
    """In-place Velocity-Verlet update (velocity_verlet.cl:88-94).

    This is the reference's own variant: the position update uses the new
    full-step velocity plus half a step of the new acceleration.
    """
    f = force.reshape(-1)
    uf, udf, uddf = u.reshape(-1), ud.reshape(-1), udd.reshape(-1)
    bt = np.asarray(bc_types).reshape(-1)
    bv = np.asarray(bc_values, dtype=np.float64).reshape(-1)
    rho = np.asarray(densities, dtype=np.float64).reshape(-1)
    half = dt / 2
    ud1 = udf + half * uddf
    udd1 = (f - damping * ud1) / rho
    udf[:] = ud1 + half * udd1
    uddf[:] = udd1
    uf[:] = np.where(bt == 0, uf + dt * (udf + half * udd1), bc_scale * bv)


class Stepper:
    """Host-resident state machine for whole simulations.

    Mirrors the per-step call sequence of ``EulerCL.__call__``,
    ``EulerCromerCL.__call__`` and ``VelocityVerletCL.__call__``
    (``peripy/integrators.py:484-503, 586-606, 700-720``): one bond-force
    pass then one displacement update, with ``write`` running the damage
    kernel (``integrators.py:285-300``).

    :arg str integrator: ``"euler"``, ``"euler_cromer"`` or
        ``"velocity_verlet"``.
    """

    def __init__(self, integrator, dt, coords, volume, family, nlist,
                 bc_types, bc_values, force_bc_types, force_bc_values,
                 bond_stiffness, critical_stretch, damping=0.0,
                 densities=None, stiffness_corrections=None, bond_types=None,
                 regimes=None, plus_cs=None, nregimes=1, u=None, ud=None):
        self.integrator = integrator
        self.dt = dt
        self.damping = damping
        self.r0 = np.asarray(coords, dtype=np.float64)
        self.vols = np.asarray(volume, dtype=np.float64)
        self.family = np.asarray(family, dtype=np.intc)
        self.nlist = np.array(nlist, dtype=np.intc, copy=True)
        n = self.r0.shape[0]
        self.bc_types = bc_types
        self.bc_values = bc_values
        self.fc_types = force_bc_types
        self.fc_values = force_bc_values
        self.k = bond_stiffness
        self.s0 = critical_stretch
        self.densities = densities
        self.sc = stiffness_corrections
        self.bond_types = bond_types
        self.nregimes = nregimes
        self.plus_cs = plus_cs
        if bond_types is not None:
            self.regimes = (np.zeros(self.nlist.shape, dtype=np.intc)
                            if regimes is None else
                            np.array(regimes, dtype=np.intc, copy=True))
        else:
            self.regimes = None
        self.u = (np.zeros((n, 3)) if u is None
                  else np.array(u, dtype=np.float64, copy=True))
        self.ud = (np.zeros((n, 3)) if ud is None
                   else np.array(ud, dtype=np.float64, copy=True))
        self.udd = np.zeros((n, 3))
        self.force = np.zeros((n, 3))
        self.body_force = np.zeros((n, 3))

    def step(self, displacement_bc_magnitude, force_bc_magnitude):
        self.force, self.body_force = bond_force(
            self.u, self.r0, self.vols, self.nlist, self.fc_types,
            self.fc_values, force_bc_magnitude, self.k, self.s0,
            self.sc, self.bond_types, self.regimes, self.plus_cs,
            self.nregimes)
        if self.integrator == "euler":
            update_euler(self.force, self.u, self.bc_types, self.bc_values,
                         displacement_bc_magnitude, self.dt)
        elif self.integrator == "euler_cromer":
            update_euler_cromer(
                self.force, self.u, self.ud, self.udd, self.bc_types,
                self.bc_values, self.densities, displacement_bc_magnitude,
                self.damping, self.dt)
        elif self.integrator == "velocity_verlet":
            update_velocity_verlet(
                self.force, self.u, self.ud, self.udd, self.bc_types,
                self.bc_values, self.densities, displacement_bc_magnitude,
                self.damping, self.dt)
        else:
            raise ValueError(self.integrator)

    def write(self):
        n_neigh, dmg = damage(self.nlist, self.family)
        return (self.u.copy(), self.ud.copy(), self.udd.copy(),
                self.force.copy(), self.body_force.copy(), dmg,
                self.nlist.copy(), n_neigh)
