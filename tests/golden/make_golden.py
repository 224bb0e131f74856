"""Build the golden fixtures in this directory from the reference's test data.

Run where the reference checkout (read-only) is available: its directory is
the first argument, else ``$PP_REFERENCE``, else ``reference`` beside this
repository's checkout::

    python tests/golden/make_golden.py [path/to/reference]

It reads the regression inputs and expected outputs that the reference's own
tests load (``peripy/test/data``, used by ``peripy/test/test_integrators.py``
``test_call`` for Euler, EulerCL, EulerCromerCL and VelocityVerletCL,
``peripy/test/test_model.py:1566-1626`` and ``conftest.py:23-63``) and stores
them, unchanged in value, as compressed ``.npz`` fixtures, so that the GPU
tests can run where the reference checkout is absent.

Outputs:

``plate2113.npz``  the 2113-node 2-D plate: mesh points and cells,
                   expected volume, the basic CL connectivity (before the
                   crack), and the expected state after 10 steps of each CL
                   integrator (Euler: u, force, damage, nlist, n_neigh;
                   Euler-Cromer adds ud; Velocity-Verlet adds ud, udd);
                   and the Cython integrator's compact connectivity before
                   the crack and after the crack and 10 steps
                   (``test_integrators.py:150-195``).
``force3.npz``     the three-node mesh of the force test.
"""
import os
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from probabilistic_peridynamics_gb300.mesh import read_vtk  # noqa: E402


def main(reference_root):
    data = pathlib.Path(reference_root) / "peripy" / "test" / "data"
    mesh = read_vtk(data / "example_mesh.vtk")
    basic = np.load(data / "expected_connectivity_basic_cl.npz")
    crack = np.load(data / "expected_connectivity_crack_cl.npz")
    ec_conn = np.load(data / "expected_connectivity_euler_cromer_cl.npz")
    vv_conn = np.load(data / "expected_connectivity_velocity_verlet_cl.npz")
    cy_basic = np.load(data / "expected_connectivity_basic.npz")
    cy_crack = np.load(data / "expected_connectivity_crack.npz")
    out = dict(
        points=mesh.points,
        cells_triangle=mesh.cells_dict["triangle"].astype(np.int32),
        cells_line=mesh.cells_dict["line"].astype(np.int32),
        volume=np.load(data / "expected_volume.npy"),
        nlist_basic=basic["nlist"], n_neigh_basic=basic["n_neigh"],
        euler_u=np.load(data / "expected_displacements.npy"),
        euler_force=np.load(data / "expected_force.npy"),
        euler_damage=np.load(data / "expected_damage.npy"),
        euler_nlist=crack["nlist"], euler_n_neigh=crack["n_neigh"],
        ec_u=np.load(data / "expected_displacements_euler_cromer.npy"),
        ec_ud=np.load(data / "expected_velocities_euler_cromer.npy"),
        ec_force=np.load(data / "expected_force_euler_cromer.npy"),
        ec_damage=np.load(data / "expected_damage_euler_cromer.npy"),
        ec_nlist=ec_conn["nlist"], ec_n_neigh=ec_conn["n_neigh"],
        vv_u=np.load(data / "expected_displacements_velocity_verlet.npy"),
        vv_ud=np.load(data / "expected_velocities_velocity_verlet.npy"),
        vv_udd=np.load(data / "expected_accelerations_velocity_verlet.npy"),
        vv_force=np.load(data / "expected_force_velocity_verlet.npy"),
        vv_damage=np.load(data / "expected_damage_velocity_verlet.npy"),
        vv_nlist=vv_conn["nlist"], vv_n_neigh=vv_conn["n_neigh"],
        # the Cython integrator's compact layout (0-padded, width 68):
        # before the crack, and after the crack and 10 Euler steps
        cy_nlist_basic=cy_basic["nlist"], cy_n_neigh_basic=cy_basic["n_neigh"],
        cy_nlist_crack=cy_crack["nlist"], cy_n_neigh_crack=cy_crack["n_neigh"],
    )
    np.savez_compressed(HERE / "plate2113.npz", **out)
    force_mesh = read_vtk(data / "force_test.vtk")
    np.savez_compressed(HERE / "force3.npz", points=force_mesh.points)
    print("wrote", HERE / "plate2113.npz", HERE / "force3.npz")


if __name__ == "__main__":
    default = (os.environ.get("PP_REFERENCE")
               or HERE.parent.parent.parent / "reference")
    main(sys.argv[1] if len(sys.argv) > 1 else default)
