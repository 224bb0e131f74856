"""Peridynamics model: ``Model`` and ``Model.simulate``.

Same constructor and ``simulate`` signatures, argument checks, exceptions
and return values as PeriPy's ``peripy/model.py:24-1575``; the time step
itself runs in the integrator (``integrators.py``).  Host-side differences,
all outside the time step:

* meshes are read with the legacy-VTK and Gmsh MSH 2.x readers of
  :mod:`.mesh` (meshio is not a dependency);
* the neighbour search runs on the GPU for CUDA integrators
  (:mod:`.neighbours`: a cell grid, one warp per node) and with
  ``scipy.spatial.cKDTree.query_pairs`` otherwise, instead of
  ``sklearn.neighbors.KDTree.query_radius`` (``model.py:564-566``); the
  neighbour *sets* are the same (distance <= horizon), rows are in
  ascending node order; the initial crack is cut on the same GPU
  (``pp_create_crack``) with the reference's swap-remove result;
* ``write_path`` caches arrays as ``.npy`` files instead of HDF5;
* the stiffness-correction algorithms (``correction.pyx``) run on the GPU
  of the CUDA integrator (:mod:`.corrections`);
* with a CUDA integrator, a write step before the last one computes the
  recorded sums on the device, bit-identical to the reference's NumPy sums
  (:mod:`.writes`), and brings back only ``u`` and ``damage`` for the mesh
  file; the last write returns the full state as the reference's does.
"""
from collections import namedtuple
import pathlib
import warnings

import numpy as np

from .integrators import Integrator
from .mesh import read_mesh, write_vtk

_MeshElements = namedtuple("MeshElements", ["connectivity", "boundary"])
_mesh_elements_2d = _MeshElements(connectivity="triangle", boundary="line")
_mesh_elements_3d = _MeshElements(connectivity="tetra", boundary="triangle")


def _progress(iterable, **kwargs):
    try:
        from tqdm import tqdm
    except ImportError:
        return iterable
    return tqdm(iterable, **kwargs)


def write_array(write_path, name, array):
    """Cache ``array`` as ``<write_path>/<name>.npy``."""
    path = pathlib.Path(write_path)
    path.mkdir(parents=True, exist_ok=True)
    np.save(path / f"{name}.npy", array)


def read_array(read_path, name):
    """Read an array cached by :func:`write_array`, or None if absent."""
    path = pathlib.Path(read_path) / f"{name}.npy"
    return np.load(path) if path.exists() else None


def neighbour_pairs(coords, horizon):
    """All unordered node pairs (i < j) with ``|r_i - r_j| <= horizon``."""
    from scipy.spatial import cKDTree
    tree = cKDTree(coords)
    pairs = tree.query_pairs(r=horizon, output_type="ndarray")
    return pairs.astype(np.int64).reshape(-1, 2)


def build_family(nnodes, pairs, pow2=True):
    """Family, padded neighbour list and max_neighbours from unique pairs.

    Rows list neighbours in ascending order.  With ``pow2`` (device
    integrators) the width is the next power of two >= family.max() and the
    padding is -1; else the width is family.max() and the padding 0
    (``peripy/model.py:575-585``).
    """
    src = np.concatenate([pairs[:, 0], pairs[:, 1]])
    dst = np.concatenate([pairs[:, 1], pairs[:, 0]])
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    family = np.bincount(src, minlength=nnodes).astype(np.intc)
    fmax = int(family.max()) if nnodes else 0
    if pow2:
        max_neighbours = np.intc(1 << (max(fmax, 1) - 1).bit_length())
        nlist = np.full((nnodes, max_neighbours), -1, dtype=np.intc)
    else:
        max_neighbours = np.intc(fmax)
        nlist = np.zeros((nnodes, max_neighbours), dtype=np.intc)
    starts = np.zeros(nnodes + 1, dtype=np.int64)
    np.cumsum(family, out=starts[1:])
    col = np.arange(src.size, dtype=np.int64) - starts[src]
    nlist[src, col] = dst
    return family, nlist, max_neighbours


def create_crack(crack, nlist, n_neigh):
    """Remove the bond pairs in ``crack`` from the neighbour list in place.

    Restates ``peripy/create_crack.pyx:1-43``: the removed entry is replaced
    by the row's last neighbour, the vacated last slot is set to -1 and the
    count is decremented, for both ends of each pair.
    """
    crack = np.asarray(crack, dtype=np.int64).reshape(-1, 2)
    for i, j in crack:
        for a, b in ((i, j), (j, i)):
            row = nlist[a]
            cnt = n_neigh[a]
            hit = np.nonzero(row[:cnt] == b)[0]
            if hit.size:
                k = hit[0]
                row[k] = row[cnt - 1]
                row[cnt - 1] = -1
                n_neigh[a] = cnt - 1


class Model(object):
    """A bond-based peridynamics model (``peripy/model.py:24``)."""

    def __init__(self, mesh_file, integrator, horizon, critical_stretch,
                 bond_stiffness, transfinite=0,
                 volume_total=None, write_path=None, connectivity=None,
                 family=None, volume=None, initial_crack=None, dimensions=2,
                 is_density=None, is_bond_type=None,
                 is_displacement_boundary=None, is_force_boundary=None,
                 is_tip=None, density=None, bond_types=None,
                 stiffness_corrections=None,
                 surface_correction=None, volume_correction=None,
                 micromodulus_function=None, node_radius=None):
        """Create a :class:`Model` object (``peripy/model.py:42-479``)."""
        if not isinstance(integrator, Integrator):
            raise InvalidIntegrator(integrator)
        self.integrator = integrator

        self.write_path = (None if write_path is None
                           else pathlib.Path(write_path))
        self.dimensions = dimensions
        if dimensions == 2:
            self.mesh_elements = _mesh_elements_2d
        elif dimensions == 3:
            self.mesh_elements = _mesh_elements_3d
        else:
            raise DimensionalityError(dimensions)

        self._read_mesh(mesh_file, transfinite)

        if volume is None:
            this_may_take_a_while(self.nnodes, 'volume')
            self.volume = self._volume(transfinite, volume_total)
            if self.write_path is not None:
                write_array(self.write_path, "volume", self.volume)
        elif type(volume) == np.ndarray:
            if np.shape(volume) != (self.nnodes, ):
                raise ValueError("volume shape is wrong, and must be "
                                 "(nnodes, ) (expected {}, got {})".format(
                                     (self.nnodes, ), np.shape(volume)))
            warnings.warn("Reading volume from argument.")
            self.volume = volume.astype(np.float64)
        else:
            raise TypeError("volume type is wrong (expected {}, got "
                            "{})".format(type(volume), np.ndarray))

        if volume_correction is not None:
            if not ((type(node_radius) == float)
                    or (type(node_radius) == np.float64)):
                raise TypeError(
                    "If volume_correction (= {}) is applied, an average node "
                    "radius must be supplied as the keyword argument "
                    "node_radius (expected {}, got {})".format(
                        volume_correction, float, type(node_radius)))
            self.horizon = horizon + node_radius
        else:
            self.horizon = horizon

        if family is None or connectivity is None:
            this_may_take_a_while(self.nnodes, 'family, connectivity')
            (self.family, nlist, n_neigh,
             self.max_neighbours) = self._set_neighbour_list(
                 self.coords, self.horizon, self.nnodes, initial_crack,
                 integrator.context)
            if self.write_path is not None:
                write_array(self.write_path, "family", self.family)
                write_array(self.write_path, "nlist", nlist)
                write_array(self.write_path, "n_neigh", n_neigh)
        else:
            if type(family) == np.ndarray:
                if np.shape(family) != (self.nnodes, ):
                    raise ValueError("family shape is wrong, and must be "
                                     "(nnodes, ) (expected {}, got {})".format(
                                         (self.nnodes, ), np.shape(family)))
                warnings.warn("Reading family from argument.")
                self.family = family.astype(np.intc)
            else:
                raise TypeError("family type is wrong (expected {}, got "
                                "{})".format(type(family), np.ndarray))
            if type(connectivity) == tuple:
                if len(connectivity) != 2:
                    raise ValueError("connectivity size is wrong (expected 2,"
                                     " got {})".format(len(connectivity)))
                warnings.warn("Reading connectivity from argument.")
                nlist, n_neigh = connectivity
                nlist = nlist.astype(np.intc)
                n_neigh = n_neigh.astype(np.intc)
                self.max_neighbours = np.intc(np.shape(nlist)[1])
                if not integrator.context:
                    if self.max_neighbours != self.family.max():
                        raise ValueError(
                            "max_neighbours, which is equal to the size of "
                            "axis 1 of nlist is wrong (expected "
                            "max_neighbours = np.shape(nlist)[1] = "
                            "family.max() = {}, got {})".format(
                                self.family.max(), self.max_neighbours))
                else:
                    test = self.max_neighbours - 1
                    if self.max_neighbours & test:
                        raise ValueError(
                            "max_neighbours, which is equal to the size of "
                            "axis 1 of nlist is wrong (expected "
                            "max_neighbours = np.shape(nlist)[1] = {}, got "
                            "{})".format(
                                1 << (int(self.family.max() - 1)).bit_length(),
                                self.max_neighbours))
            else:
                raise TypeError("connectivity type is wrong (expected {} or"
                                " {}, got {})".format(
                                    tuple, type(None), type(connectivity)))

        if np.any(self.family == 0):
            raise FamilyError(self.family)

        self.initial_connectivity = (nlist, n_neigh)
        self.degrees_freedom = 3

        if stiffness_corrections is None:
            # micromodulus, volume and surface factors
            # (peripy/model.py:349-375), computed on the integrator's GPU
            if ((micromodulus_function is not None
                 or volume_correction is not None
                 or surface_correction is not None)
                    and not integrator.context):
                raise NotImplementedError(
                    "stiffness corrections are computed on the GPU of a "
                    "CUDA integrator")
            from .corrections import stiffness_corrections as _corrections
            self.stiffness_corrections = _corrections(
                self.coords, self.volume, nlist, n_neigh, horizon,
                micromodulus_function=micromodulus_function,
                volume_correction=volume_correction,
                surface_correction=surface_correction,
                node_radius=node_radius, dimensions=self.dimensions,
                search_horizon=self.horizon,
                context=integrator.context if integrator.context else None)
            if (self.stiffness_corrections is not None
                    and self.write_path is not None):
                write_array(self.write_path, "stiffness_corrections",
                            self.stiffness_corrections)
        elif type(stiffness_corrections) == np.ndarray:
            if np.shape(stiffness_corrections) != (
                    self.nnodes, self.max_neighbours):
                raise ValueError("stiffness_corrections shape is wrong, "
                                 "and must be (nnodes, max_neighbours) "
                                 "(expected {}, got {})".format(
                                     (self.nnodes, self.max_neighbours),
                                     np.shape(stiffness_corrections)))
            warnings.warn("Reading stiffness_corrections from argument.")
            self.stiffness_corrections = stiffness_corrections.astype(
                np.float64)
        else:
            raise TypeError("stiffness_corrections type is wrong (expected {}"
                            ", got {})".format(np.ndarray,
                                               type(stiffness_corrections)))

        if is_bond_type is None:
            def is_bond_type(x, y):
                return 0

        (self.bond_stiffness, self.critical_stretch, self.plus_cs,
         self.nbond_types, self.nregimes) = self._set_damage_model(
             bond_stiffness, critical_stretch)

        if bond_types is None:
            self.bond_types = self._set_bond_types(
                self.initial_connectivity, is_bond_type, self.nbond_types,
                self.nregimes)
        elif type(bond_types) == np.ndarray:
            if np.shape(bond_types) != (self.nnodes, self.max_neighbours):
                raise ValueError("bond_types shape is wrong, "
                                 "and must be (nnodes, max_neighbours) "
                                 "(expected {}, got {})".format(
                                     (self.nnodes, self.max_neighbours),
                                     np.shape(bond_types)))
            warnings.warn("Reading bond_types from argument.")
            self.bond_types = bond_types.astype(np.intc)
        else:
            raise TypeError("bond_types type is wrong (expected {}"
                            ", got {})".format(np.ndarray, type(bond_types)))

        self.densities = self._set_densities(density, is_density)

        if is_force_boundary is None:
            def is_force_boundary(x):
                return [None, None, None]
        if is_displacement_boundary is None:
            def is_displacement_boundary(x):
                return [None, None, None]
        if is_tip is None:
            def is_tip(x):
                return [None, None, None]

        (self.bc_types, self.bc_values, self.force_bc_types,
         self.force_bc_values, self.tip_types,
         self.ntips) = self._set_boundary_conditions(
            is_displacement_boundary, is_force_boundary, is_tip)

        self.integrator.build(
            self.nnodes, self.degrees_freedom, self.max_neighbours,
            self.coords, self.volume, self.family, self.bc_types,
            self.bc_values, self.force_bc_types, self.force_bc_values,
            self.stiffness_corrections, self.bond_types, self.densities)

    # ------------------------------------------------------------------ mesh
    def _read_mesh(self, filename, transfinite):
        """Read nodes and cells (``peripy/model.py:481-503``)."""
        mesh = read_mesh(filename)
        self.coords = np.array(mesh.points, dtype=np.float64)
        self.nnodes = self.coords.shape[0]
        if not transfinite:
            self.mesh_connectivity = mesh.cells_dict[
                self.mesh_elements.connectivity]
            self.mesh_boundary = mesh.cells_dict.get(
                self.mesh_elements.boundary,
                np.zeros((0, 2 if self.dimensions == 2 else 3),
                         dtype=np.int64))
        else:
            self.mesh_connectivity = None
            self.mesh_boundary = None

    def write_mesh(self, filename, damage=None, displacements=None,
                   file_format=None):
        """Write nodes, cells and point data (``peripy/model.py:505-534``)."""
        cells = []
        if self.mesh_connectivity is not None:
            cells.append((self.mesh_elements.connectivity,
                          self.mesh_connectivity))
            if self.mesh_boundary is not None and len(self.mesh_boundary):
                cells.append((self.mesh_elements.boundary,
                              self.mesh_boundary))
        write_vtk(filename, self.coords, cells,
                  {"damage": damage, "displacements": displacements})

    def _set_neighbour_list(self, coords, horizon, nnodes,
                            initial_crack=None, context=None):
        """Family, neighbour list and crack (``peripy/model.py:536-597``).

        With a CUDA integrator the families are built and the initial crack
        is cut on its GPU (:func:`.neighbours.neighbour_family`,
        :func:`.neighbours.create_crack`), else on the host; both give the
        same rows.
        """
        if context:
            from .neighbours import neighbour_family
            family, nlist, max_neighbours = neighbour_family(
                coords, horizon, context, pow2=True)
        else:
            pairs = neighbour_pairs(coords, horizon)
            family, nlist, max_neighbours = build_family(
                nnodes, pairs, pow2=False)
        n_neigh = family.copy()
        if initial_crack is not None:
            if callable(initial_crack):
                initial_crack = initial_crack(coords, nlist, n_neigh)
            if context:
                from .neighbours import create_crack as crack_on_gpu
                crack_on_gpu(np.array(initial_crack, dtype=np.int32), nlist,
                             n_neigh, context)
            else:
                create_crack(np.array(initial_crack, dtype=np.int32), nlist,
                             n_neigh)
        return (family, nlist, n_neigh, max_neighbours)

    def _volume(self, transfinite, volume_total):
        """Node volumes (areas) from the cells (``peripy/model.py:599-655``).

        Each element's volume is split equally among its nodes and
        accumulated in element order.
        """
        if transfinite:
            if volume_total is None:
                raise TypeError("In transfinite mode, a total mesh volume "
                                "volume_total' must be provided as a keyword"
                                " argument (expected {}, got {})".format(
                                    float, type(volume_total)))
            return (volume_total / self.nnodes) * np.ones(self.nnodes)
        volume = np.zeros(self.nnodes)
        cells = np.asarray(self.mesh_connectivity, dtype=np.int64)
        pts = self.coords[cells]
        if self.dimensions == 2:
            c = np.cross(pts[:, 1] - pts[:, 0], pts[:, 2] - pts[:, 0])
            ev = 0.5 * np.sqrt(np.sum(c * c, axis=1))
            nodes_per = 3
        else:
            i = pts[:, 0] - pts[:, 3]
            j = pts[:, 1] - pts[:, 3]
            k = pts[:, 2] - pts[:, 3]
            ev = np.abs(np.einsum("ij,ij->i", i, np.cross(j, k))) / 6
            nodes_per = 4
        np.add.at(volume, cells.reshape(-1),
                  np.repeat(ev / nodes_per, nodes_per))
        return volume.astype(np.float64)

    def _set_densities(self, density, is_density):
        """(nnodes, 3) densities or None (``peripy/model.py:657-707``)."""
        if density is None:
            if is_density is None:
                return None
            if not callable(is_density):
                raise TypeError("is_density must be a *function*.")
            if type(is_density(self.coords[0])) is not float:
                raise TypeError(
                    "is_density must be a function that returns a *float* "
                    "(expected {}, got {})".format(
                        float, type(is_density(self.coords[0]))))
            density = np.ones(self.nnodes)
            for i in range(self.nnodes):
                density[i] = is_density(self.coords[i])
            if self.write_path is not None:
                write_array(self.write_path, "density", density)
            return np.transpose(np.tile(density, (self.degrees_freedom, 1))
                                ).astype(np.float64)
        if type(density) == np.ndarray:
            if np.shape(density) != (self.nnodes,):
                raise ValueError("densty shape is wrong, and must be "
                                 "(nnodes,) (expected {}, got {})".format(
                                     (self.nnodes,), np.shape(density)))
            warnings.warn("Reading density from argument.")
            return np.transpose(np.tile(density, (self.degrees_freedom, 1))
                                ).astype(np.float64)
        raise TypeError("density type is wrong, and must be an array of"
                        " shape (nnodes,) (expected {}, got {})".format(
                            np.ndarray, type(density)))

    def _set_bond_types(self, connectivity, is_bond_type, nbond_types,
                        nregimes):
        """Bond-type table (``peripy/model.py:709-780``)."""
        if nbond_types != 1:
            if not callable(is_bond_type):
                raise TypeError("is_bond_type must be a *function*.")
            nlist, n_neigh = connectivity
            bond_types = np.zeros((self.nnodes, self.max_neighbours))
            for i in range(self.nnodes):
                for neigh in range(n_neigh[i]):
                    j = nlist[i][neigh]
                    bond_type = is_bond_type(self.coords[i, :],
                                             self.coords[j, :])
                    if type(bond_type) is not int:
                        raise TypeError(
                            "is_bond_type must be a function that returns an "
                            "*int* (expected {}, got {})".format(
                                int, type(bond_type)))
                    if bond_type < 0:
                        raise ValueError(
                            "is_bond_type must be a function that returns a "
                            "*positive* int or 0 (got {})".format(bond_type))
                    if bond_type > nbond_types - 1:
                        raise ValueError(
                            "is_bond_type must be a function that returns a "
                            "positive int or 0 which is *less* than "
                            "nbond_types (the number of different bonds, "
                            "nbond_types = {}, got is_bond_type = {} for "
                            "node coordinate pair {}, {})".format(
                                nbond_types, bond_type, self.coords[i, :],
                                self.coords[j, :]))
                    bond_types[i][neigh] = bond_type
            bond_types = bond_types.astype(np.intc)
        elif nregimes != 1:
            bond_types = np.zeros((self.nnodes, self.max_neighbours),
                                  dtype=np.intc)
        else:
            return None
        if self.write_path is not None:
            write_array(self.write_path, "bond_types", bond_types)
        return bond_types

    def _set_damage_model(self, bond_stiffness, critical_stretch):
        """Normalise the damage model (``peripy/model.py:941-1091``).

        :returns: ``(bond_stiffness, critical_stretch, plus_cs, nbond_types,
            nregimes)``; ``plus_cs[r] = plus_cs[r-1] + k[r-1]*s[r-1] -
            k[r]*s[r-1]`` so the n-linear force is continuous.
        """
        if type(bond_stiffness) != type(critical_stretch):
            raise TypeError(
                "bond_stiffness must be the same type as critical_stretch "
                "(expected {}, got {})".format(type(critical_stretch),
                                               type(bond_stiffness)))
        if type(bond_stiffness) in (list, np.ndarray):
            if np.shape(bond_stiffness) != np.shape(critical_stretch):
                raise ValueError(
                    "The shape of bond_stiffness must be equal to the shape "
                    "of critical_stretch (expected {}, got {})".format(
                        np.shape(critical_stretch), np.shape(bond_stiffness)))
            if np.shape(bond_stiffness) == (1,):
                nregimes = 1
                nbond_types = 1
                bond_stiffness = np.float64(bond_stiffness[0])
                critical_stretch = np.float64(critical_stretch[0])
                plus_cs = None
            elif np.shape(bond_stiffness) == ():
                nregimes = 1
                nbond_types = 1
                bond_stiffness = np.float64(bond_stiffness)
                critical_stretch = np.array(critical_stretch)
                plus_cs = None
            elif np.shape(bond_stiffness[0]) == (1,):
                nregimes = 1
                nbond_types = np.shape(bond_stiffness)[0]
                bond_stiffness = np.array(bond_stiffness, dtype=np.float64)
                critical_stretch = np.array(critical_stretch,
                                            dtype=np.float64)
                plus_cs = np.zeros(nbond_types).astype(np.float64)
            elif np.shape(bond_stiffness[0]) == ():
                nbond_types = 1
                nregimes = np.shape(bond_stiffness)[0]
                if not all(critical_stretch[i] <= critical_stretch[i + 1]
                           for i in range(nregimes - 1)):
                    raise DamageModelError(critical_stretch)
                bond_stiffness = np.array(bond_stiffness, dtype=np.float64)
                critical_stretch = np.array(critical_stretch,
                                            dtype=np.float64)
                plus_cs = np.zeros(nregimes)
                c_prev = 0.0
                plus_cs[0] = c_prev
                for r in range(1, nregimes):
                    c_i = (c_prev
                           + (bond_stiffness[r - 1] * critical_stretch[r - 1])
                           - (bond_stiffness[r] * critical_stretch[r - 1]))
                    plus_cs[r] = c_i
                    c_prev = c_i
                plus_cs = plus_cs.astype(np.float64)
            else:
                nregimes = np.shape(bond_stiffness)[1]
                nbond_types = np.shape(bond_stiffness)[0]
                for i in range(nbond_types):
                    if not all(critical_stretch[i][j] <=
                               critical_stretch[i][j + 1]
                               for j in range(nregimes - 1)):
                        raise DamageModelError(critical_stretch[i])
                bond_stiffness = np.array(bond_stiffness, dtype=np.float64)
                critical_stretch = np.array(critical_stretch,
                                            dtype=np.float64)
                plus_cs = np.zeros((nbond_types, nregimes))
                c_prev = np.zeros(nbond_types)
                plus_cs[:, 0] = c_prev
                for r in range(1, nregimes):
                    c_i = (c_prev
                           + (bond_stiffness[:, r - 1] *
                              critical_stretch[:, r - 1])
                           - (bond_stiffness[:, r] *
                              critical_stretch[:, r - 1]))
                    plus_cs[:, r] = c_i
                    c_prev = c_i
                plus_cs = plus_cs.astype(np.float64)
        elif type(bond_stiffness) in (float, np.float64):
            nregimes = 1
            nbond_types = 1
            bond_stiffness = np.float64(bond_stiffness)
            critical_stretch = np.float64(critical_stretch)
            plus_cs = None
        else:
            raise TypeError(
                "Type of bond_stiffness and critical_stretch is not supported "
                "(expected {} or {}, got {})".format(
                    float, np.ndarray, type(bond_stiffness)))
        nregimes = np.intc(nregimes)
        nbond_types = np.intc(nbond_types)
        if np.any(critical_stretch < 0):
            raise ValueError("critical_stretch values must not be < 0, "
                             "(got {})".format(critical_stretch))
        return (bond_stiffness, critical_stretch, plus_cs, nbond_types,
                nregimes)

    def _set_boundary_conditions(self, is_displacement_boundary,
                                 is_force_boundary, is_tip):
        """BC arrays and tip lists (``peripy/model.py:1093-1212``)."""
        functions = {'is_displacement_boundary': is_displacement_boundary,
                     'is_force_boundary': is_force_boundary,
                     'is_tip': is_tip}
        for function in functions:
            if not callable(functions[function]):
                raise TypeError("{} must be a *function*.".format(function))
            if type(functions[function](self.coords[0][:])) is not list:
                raise TypeError(
                    "{} must be a function that returns a *list*.".format(
                        function))
            if len(functions[function](self.coords[0][:])) != 3:
                if function == 'is_tip':
                    raise TypeError("{} must be a function that returns a list"
                                    " of length *3* of ints or strings or "
                                    "tuples of ints or strings")
                raise TypeError("{} must be a function that returns a list"
                                " of length *3* of floats or None")

        def set_tip(tip, i, j, tip_types, ntips):
            if str(tip) not in ntips:
                ntips[str(tip)] = 0
                tip_types[str(tip)] = []
            ntips[str(tip)] += 1
            tip_types[str(tip)].append((i, j))
            return tip_types, ntips

        n = self.nnodes
        bc_types = np.zeros((n, self.degrees_freedom), dtype=np.intc)
        bc_values = np.zeros((n, self.degrees_freedom), dtype=np.float64)
        force_bc_types = np.zeros((n, self.degrees_freedom), dtype=np.intc)
        force_bc_values = np.zeros((n, self.degrees_freedom),
                                   dtype=np.float64)
        tip_types = {}
        num_force_bc_nodes = 0
        ntips = {'model': n}
        for i in range(n):
            bnd = is_displacement_boundary(self.coords[i][:])
            forces_bnd = is_force_boundary(self.coords[i][:])
            tip = is_tip(self.coords[i][:])
            is_force_node = 0
            for j in range(self.degrees_freedom):
                forces_bnd_j = forces_bnd[j]
                bnd_j = bnd[j]
                tip_j = tip[j]
                if bnd_j is not None:
                    bc_types[i, j] = np.intc(1)
                    bc_values[i, j] = np.float64(bnd_j)
                if forces_bnd_j is not None:
                    is_force_node = 1
                    force_bc_types[i, j] = np.intc(1)
                    force_bc_values[i, j] = np.float64(
                        forces_bnd_j / self.volume[i])
                if tip_j is not None:
                    if type(tip_j) is tuple:
                        for tip_jk in tip_j:
                            tip_types, ntips = set_tip(tip_jk, i, j,
                                                       tip_types, ntips)
                    else:
                        tip_types, ntips = set_tip(tip_j, i, j, tip_types,
                                                   ntips)
            num_force_bc_nodes += is_force_node
        if num_force_bc_nodes != 0:
            force_bc_values = np.float64(
                np.divide(force_bc_values, num_force_bc_nodes))
        return (bc_types, bc_values, force_bc_types, force_bc_values,
                tip_types, ntips)

    # -------------------------------------------------------------- simulate
    def simulate(self, steps, u=None, ud=None, connectivity=None,
                 regimes=None, critical_stretch=None, bond_stiffness=None,
                 displacement_bc_magnitudes=None, force_bc_magnitudes=None,
                 first_step=1, write=None, write_path=None):
        """Simulate the model (``peripy/model.py:1214-1385``).

        :returns: ``(u, damage, (nlist, n_neigh), force, ud, data)``.
        """
        (u, ud, udd, force, body_force, nlist, n_neigh,
         displacement_bc_magnitudes, force_bc_magnitudes, damage, data,
         nwrites, write_path) = self._simulate_initialise(
             steps, first_step, write, regimes, u, ud,
             displacement_bc_magnitudes, force_bc_magnitudes, connectivity,
             bond_stiffness, critical_stretch, write_path)

        run = getattr(self.integrator, "_run", None)
        sums = None
        if write and getattr(self.integrator, "write_sums", None) is not None:
            from .writes import WriteSums
            sums = WriteSums(self.integrator.context, self.nnodes,
                             self.integrator.vols_d, self.tip_types)
        step = first_step
        last = first_step + steps - 1
        bar = _progress(range(steps), desc="Simulation Progress",
                        unit="steps")
        # A write with device sums leaves its mesh file and record pending
        # until the next segment of steps is queued, so that the host writes
        # the file while the GPU steps; it is finished before the next write
        # refills u and damage.
        pending = None
        while step <= last:
            if write:
                nxt = min(last, ((step + write - 1) // write) * write)
            else:
                nxt = last
            count = nxt - step + 1
            if run is not None:
                run(displacement_bc_magnitudes, force_bc_magnitudes,
                    step - 1, count)
            else:
                for s in range(step, nxt + 1):
                    self.integrator(displacement_bc_magnitudes[s - 1],
                                    force_bc_magnitudes[s - 1])
            if pending is not None:
                self._finish_write(data, nwrites, *pending)
                pending = None
            step = nxt + 1
            if hasattr(bar, "update"):
                bar.update(count)
            if write and nxt % write == 0:
                ii = nxt // write - (first_step - 1) // write - 1
                if sums is not None:
                    u, damage, values = self.integrator.write_sums(
                        u, damage, sums)
                    pending = (write_path / f"U_{nxt}.vtk", u, damage, ii,
                               nxt, values)
                    continue
                (u, ud, udd, force, body_force, damage, nlist,
                 n_neigh) = self.integrator.write(
                     u, ud, udd, body_force, force, damage, nlist, n_neigh)
                self.write_mesh(write_path / f"U_{nxt}.vtk", damage, u)
                self._record(data, ii, nxt, nwrites, u, ud, udd, force,
                             body_force, damage)
        if pending is not None:
            self._finish_write(data, nwrites, *pending)
        if hasattr(bar, "close"):
            bar.close()
        for tip_type_str in data:
            ntip = self.ntips[tip_type_str]
            if ntip != 0:
                data[tip_type_str]['displacement'] /= ntip
                data[tip_type_str]['velocity'] /= ntip
                data[tip_type_str]['acceleration'] /= ntip
        (u, ud, udd, force, body_force, damage, nlist,
         n_neigh) = self.integrator.write(
             u, ud, udd, force, body_force, damage, nlist, n_neigh)
        return (u, damage, (nlist, n_neigh), force, ud, data)

    def _record(self, data, ii, step, nwrites, u, ud, udd, force, body_force,
                damage):
        """Tip and model sums of one write (``peripy/model.py:1320-1366``).

        ``force`` and ``body_force`` arrive swapped, as the reference's
        intermediate ``write`` call passes and unpacks them.
        """
        for tip_type, node_list in self.tip_types.items():
            if tip_type not in data:
                data[tip_type] = {
                    key: np.zeros(nwrites, dtype=np.float64)
                    for key in ('displacement', 'velocity', 'acceleration',
                                'force', 'body_force')}
            for i, j in node_list:
                data[tip_type]['displacement'][ii] += u[i, j]
                data[tip_type]['velocity'][ii] += ud[i, j]
                data[tip_type]['acceleration'][ii] += udd[i, j]
                data[tip_type]['force'][ii] += force[i, j] * self.volume[i]
                data[tip_type]['body_force'][ii] += (
                    body_force[i, j] * self.volume[i])
        data['model']['step'][ii] = step
        data['model']['displacement'][ii] = np.sum(u)
        data['model']['velocity'][ii] = np.sum(ud)
        data['model']['acceleration'][ii] = np.sum(udd)
        data['model']['force'][ii] = np.sum(
            force * self.volume[:, np.newaxis])
        data['model']['body_force'][ii] = np.sum(
            body_force * self.volume[:, np.newaxis])
        damage_sum = np.sum(damage)
        data['model']['damage_sum'][ii] = damage_sum
        if damage_sum > 0.05 * self.nnodes:
            warnings.warn('Over 5% of bonds have broken! peridynamics '
                          'simulation continuing')

    def _finish_write(self, data, nwrites, path, u, damage, ii, step,
                      values):
        """Mesh file and record of a write with device sums."""
        self.write_mesh(path, damage, u)
        self._record_sums(data, ii, step, nwrites, values)

    def _record_sums(self, data, ii, step, nwrites, values):
        """:meth:`_record` from sums computed on the device
        (:class:`.writes.WriteSums`, bit-identical to the NumPy sums)."""
        from .writes import TIP_KEYS
        for t, tip_type in enumerate(self.tip_types):
            if tip_type not in data:
                data[tip_type] = {
                    key: np.zeros(nwrites, dtype=np.float64)
                    for key in TIP_KEYS}
            for q, key in enumerate(TIP_KEYS):
                data[tip_type][key][ii] += values[6 + 5 * t + q]
        data['model']['step'][ii] = step
        (data['model']['displacement'][ii], data['model']['velocity'][ii],
         data['model']['acceleration'][ii], data['model']['force'][ii],
         data['model']['body_force'][ii]) = values[:5]
        damage_sum = values[5]
        data['model']['damage_sum'][ii] = damage_sum
        if damage_sum > 0.05 * self.nnodes:
            warnings.warn('Over 5% of bonds have broken! peridynamics '
                          'simulation continuing')

    def _simulate_initialise(self, steps, first_step, write, regimes, u, ud,
                             displacement_bc_magnitudes, force_bc_magnitudes,
                             connectivity, bond_stiffness, critical_stretch,
                             write_path):
        """Initialise simulation variables (``peripy/model.py:1387-1575``)."""
        if u is None:
            u = np.zeros((self.nnodes, 3), dtype=np.float64)
        if ud is None:
            ud = np.zeros((self.nnodes, 3), dtype=np.float64)
        force = np.zeros((self.nnodes, 3), dtype=np.float64)
        body_force = np.zeros((self.nnodes, 3), dtype=np.float64)
        damage = np.zeros(self.nnodes, dtype=np.float64)
        udd = np.zeros((self.nnodes, 3), dtype=np.float64)
        if displacement_bc_magnitudes is None:
            displacement_bc_magnitudes = np.zeros(first_step + steps - 1,
                                                  dtype=np.float64)
        elif type(displacement_bc_magnitudes) == np.ndarray:
            if len(displacement_bc_magnitudes) < steps:
                raise ValueError("displacement_bc_magnitudes length must be "
                                 "equal to or greater than (first_step + steps"
                                 " - 1), (expected {}, got {})".format(
                                     first_step + steps - 1,
                                     len(displacement_bc_magnitudes)))
            displacement_bc_magnitudes = displacement_bc_magnitudes.astype(
                np.float64)
        else:
            raise TypeError("displacement_bc_magnitudes type is wrong "
                            "(expected {}, got {})".format(
                                np.ndarray,
                                type(displacement_bc_magnitudes)))
        if force_bc_magnitudes is None:
            force_bc_magnitudes = np.zeros(first_step + steps - 1,
                                           dtype=np.float64)
        elif type(force_bc_magnitudes) == np.ndarray:
            if len(force_bc_magnitudes) < steps:
                raise ValueError("force_bc_magnitudes length must be "
                                 "equal to or greater than (first_step + steps"
                                 " - 1), (expected {}, got {})".format(
                                     first_step + steps - 1,
                                     len(force_bc_magnitudes)))
            force_bc_magnitudes = force_bc_magnitudes.astype(np.float64)
        else:
            raise TypeError("force_bc_magnitudes type is wrong "
                            "(expected {}, got {})".format(
                                np.ndarray, type(force_bc_magnitudes)))
        if connectivity is None:
            nlist, n_neigh = self.initial_connectivity
            nlist = nlist.copy()
            n_neigh = n_neigh.copy()
        elif type(connectivity) == tuple:
            if len(connectivity) != 2:
                raise ValueError("connectivity size is wrong (expected 2,"
                                 " got {})".format(len(connectivity)))
            nlist, n_neigh = connectivity
        else:
            raise TypeError("connectivity type is wrong (expected {} or"
                            " {}, got {})".format(tuple, type(None),
                                                  type(connectivity)))
        if regimes is None:
            regimes = np.zeros((self.nnodes, self.max_neighbours),
                               dtype=np.intc)
        elif type(regimes) == np.ndarray:
            if np.shape(regimes) != (self.nnodes, self.max_neighbours):
                raise ValueError("regimes shape is wrong, and must be "
                                 "(nnodes, max_neighbours) "
                                 "(expected {}, got {})".format(
                                     (self.nnodes, self.max_neighbours),
                                     np.shape(regimes)))
            regimes = regimes.astype(np.intc)
        else:
            raise TypeError("regimes type is wrong "
                            "(expected {} or {}, got {})".format(
                                np.ndarray, type(None), type(regimes)))
        if (bond_stiffness is None) and (critical_stretch is None):
            bond_stiffness = self.bond_stiffness
            critical_stretch = self.critical_stretch
            plus_cs = self.plus_cs
            nbond_types = self.nbond_types
            nregimes = self.nregimes
        else:
            (bond_stiffness, critical_stretch, plus_cs, nbond_types,
             nregimes) = self._set_damage_model(bond_stiffness,
                                                critical_stretch)
            if nbond_types != self.nbond_types:
                raise ValueError(
                    "Number of bond types has unexpectedly changed from when "
                    " the model was constructed. Please reinstantiate "
                    ":class:`Model` with the new number of bond types "
                    "(expected {}, got {}).".format(self.nbond_types,
                                                    nbond_types))
        write_path = (pathlib.Path() if write_path is None
                      else pathlib.Path(write_path))
        data = {}
        nwrites = None
        if write:
            nwrites = ((first_step + steps - 1) // write
                       - (first_step - 1) // write)
            data['model'] = {
                'step': np.zeros(nwrites, dtype=int),
                'displacement': np.zeros(nwrites, dtype=np.float64),
                'velocity': np.zeros(nwrites, dtype=np.float64),
                'acceleration': np.zeros(nwrites, dtype=np.float64),
                'force': np.zeros(nwrites, dtype=np.float64),
                'body_force': np.zeros(nwrites, dtype=np.float64),
                'damage_sum': np.zeros(nwrites, dtype=np.float64)}
        self.integrator.create_buffers(
            nlist, n_neigh, bond_stiffness, critical_stretch, plus_cs, u, ud,
            udd, force, body_force, damage, regimes, nregimes, nbond_types)
        return (u, ud, udd, force, body_force, nlist, n_neigh,
                displacement_bc_magnitudes, force_bc_magnitudes, damage, data,
                nwrites, write_path)


def initial_crack_helper(crack_function):
    """Build an ``initial_crack`` function (``peripy/model.py:1578-1612``).

    ``crack_function(icoord, jcoord)`` returns a truthy value where a bonded
    pair (i < j) crosses the crack.
    """
    def initial_crack(coords, nlist, n_neigh):
        crack = []
        nnodes = nlist.shape[0]
        pairs = [(i, j) for i in range(nnodes) for j in nlist[i][0:n_neigh[i]]
                 if i < j]
        for i, j in pairs:
            if crack_function(coords[i], coords[j]):
                crack.append((i, j))
        return crack
    return initial_crack


def this_may_take_a_while(nnodes, calculation):
    """Warn when nnodes is large (``peripy/model.py:1615-1630``)."""
    if nnodes > 9000:
        warnings.warn(f"Calculating {calculation} for {nnodes} nodes... "
                      "this may take a while.")


class DimensionalityError(Exception):
    """An invalid dimensionality argument used to construct a model."""

    def __init__(self, dimensions):
        super().__init__("The number of dimensions must be 2 or 3,"
                         f" {dimensions} was given.")


class FamilyError(Exception):
    """One or more nodes have no bonds in the initial state."""

    def __init__(self, family):
        indicies = " ".join(f"{index}" for index in np.where(family == 0)[0])
        super().__init__("The following nodes have no bonds in the initial "
                         f"state, {indicies}.")


class DamageModelError(Exception):
    """An invalid critical stretch argument was used to construct a model."""

    def __init__(self, critical_stretch):
        super().__init__(
            "The critical_stretch list or array for a bond-type with "
            "multiple regimes must be in ascending order, "
            f" {critical_stretch} was given.")


class InvalidIntegrator(Exception):
    """An invalid integrator has been passed to `simulate`."""

    def __init__(self, integrator):
        super().__init__(f"{integrator} is not an instance of "
                         "probabilistic_peridynamics_gb300.integrators."
                         "Integrator")
