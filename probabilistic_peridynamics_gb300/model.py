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



def _given_array(name, value, shape, dtype, shape_text):
    """An array a caller supplied in place of one :class:`Model` would
    compute: its type and shape are checked, its use is announced with a
    warning (as PeriPy announces it) and it is converted to ``dtype``."""
    if type(value) != np.ndarray:
        raise TypeError("{} type is wrong (expected {}, got {})".format(
            name, np.ndarray, type(value)))
    if np.shape(value) != shape:
        raise ValueError("{} shape is wrong, and must be {} (expected {}, "
                         "got {})".format(name, shape_text, shape,
                                          np.shape(value)))
    warnings.warn("Reading {} from argument.".format(name))
    return value.astype(dtype)


def _connectivity_pair(connectivity):
    """``(nlist, n_neigh)`` from a connectivity argument (a 2-tuple)."""
    if type(connectivity) != tuple:
        raise TypeError("connectivity type is wrong (expected {} or {}, got "
                        "{})".format(tuple, type(None), type(connectivity)))
    if len(connectivity) != 2:
        raise ValueError("connectivity size is wrong (expected 2, got "
                         "{})".format(len(connectivity)))
    return connectivity


def _schedule(name, value, first_step, steps):
    """Per-step boundary-condition magnitudes: zeros by default, else a
    float64 copy of an array that covers ``steps`` steps."""
    last = first_step + steps - 1
    if value is None:
        return np.zeros(last, dtype=np.float64)
    if type(value) != np.ndarray:
        raise TypeError("{} type is wrong (expected {}, got {})".format(
            name, np.ndarray, type(value)))
    if len(value) < steps:
        raise ValueError("{} length must be equal to or greater than "
                         "(first_step + steps - 1), (expected {}, got "
                         "{})".format(name, last, len(value)))
    return value.astype(np.float64)


class DamageModel(tuple):
    """``(bond_stiffness, critical_stretch, plus_cs, nbond_types,
    nregimes)`` of a normalised damage model (see :func:`damage_model`)."""

    __slots__ = ()


def _nlinear(k, s):
    """Tables of an n-linear model, rows = bond types: the stretches of a
    row must not decrease; ``plus_cs`` keeps the force continuous across
    regimes (``plus_cs[:, r] = plus_cs[:, r-1] + k[:, r-1] s[:, r-1] -
    k[:, r] s[:, r-1]``, peripy/model.py:1031-1039)."""
    for row in s:
        if not np.all(row[:-1] <= row[1:]):  # NaN fails too
            raise DamageModelError(row)
    from .pointset import nlinear_tables
    return nlinear_tables(k, s)[2]


#: How each layout of (bond_stiffness, critical_stretch) is normalised:
#: (number of bond types, number of regimes, builder of (k, s, plus_cs)).
#: Layouts: a Python or NumPy float; an array of shape (1,); a 0-d array;
#: one stiffness per bond type (shape (T, 1)); one bond type with R
#: regimes (shape (R,)); T bond types with R regimes (shape (T, R)).
_DAMAGE_LAYOUTS = {
    "scalar": (lambda k: 1, lambda k: 1,
               lambda k, s: (np.float64(k), np.float64(s), None)),
    "single": (lambda k: 1, lambda k: 1,
               lambda k, s: (np.float64(k[0]), np.float64(s[0]), None)),
    "0d": (lambda k: 1, lambda k: 1,
           lambda k, s: (np.float64(k), np.array(s), None)),
    "types": (lambda k: len(k), lambda k: 1,
              lambda k, s: (np.array(k, dtype=np.float64),
                            np.array(s, dtype=np.float64),
                            np.zeros(len(k), dtype=np.float64))),
    "regimes": (lambda k: 1, lambda k: len(k),
                lambda k, s: (np.array(k, dtype=np.float64),
                              np.array(s, dtype=np.float64),
                              _nlinear(np.array([k], dtype=np.float64),
                                       np.array([s], dtype=np.float64))[0])),
    "table": (lambda k: np.shape(k)[0], lambda k: np.shape(k)[1],
              lambda k, s: (np.array(k, dtype=np.float64),
                            np.array(s, dtype=np.float64),
                            _nlinear(np.array(k, dtype=np.float64),
                                     np.array(s, dtype=np.float64)))),
}


def _damage_layout(bond_stiffness, critical_stretch):
    if type(bond_stiffness) != type(critical_stretch):
        raise TypeError(
            "bond_stiffness must be the same type as critical_stretch "
            "(expected {}, got {})".format(type(critical_stretch),
                                           type(bond_stiffness)))
    if type(bond_stiffness) in (float, np.float64):
        return "scalar"
    if type(bond_stiffness) not in (list, np.ndarray):
        raise TypeError(
            "Type of bond_stiffness and critical_stretch is not supported "
            "(expected {} or {}, got {})".format(float, np.ndarray,
                                                  type(bond_stiffness)))
    shape = np.shape(bond_stiffness)
    if shape != np.shape(critical_stretch):
        raise ValueError(
            "The shape of bond_stiffness must be equal to the shape of "
            "critical_stretch (expected {}, got {})".format(
                np.shape(critical_stretch), shape))
    if shape == (1,):
        return "single"
    if shape == ():
        return "0d"
    inner = np.shape(bond_stiffness[0])
    if inner == (1,):
        return "types"
    return "regimes" if inner == () else "table"


def damage_model(bond_stiffness, critical_stretch):
    """Normalise a damage model as PeriPy's ``Model`` takes it
    (``peripy/model.py:941-1091``): a float (PMB), or arrays of stiffness
    and critical stretch per bond type and/or regime (n-linear).

    :returns: :class:`DamageModel` ``(bond_stiffness, critical_stretch,
        plus_cs, nbond_types, nregimes)``: scalars (``plus_cs`` None) for
        one type and one regime, else float64 tables; the counts as
        ``np.intc``.
    """
    ntypes, nregimes, build = _DAMAGE_LAYOUTS[
        _damage_layout(bond_stiffness, critical_stretch)]
    k, s, plus_cs = build(bond_stiffness, critical_stretch)
    if np.any(s < 0):
        raise ValueError("critical_stretch values must not be < 0, "
                         "(got {})".format(s))
    return DamageModel((k, s, plus_cs, np.intc(ntypes(bond_stiffness)),
                        np.intc(nregimes(bond_stiffness))))


def _check_node_function(name, function, x):
    """A user function of a node's coordinates must return a list of 3."""
    if not callable(function):
        raise TypeError("{} must be a *function*.".format(name))
    value = function(x)
    if type(value) is not list:
        raise TypeError("{} must be a function that returns a *list*."
                        .format(name))
    if len(value) != 3:
        if name == 'is_tip':
            raise TypeError("{} must be a function that returns a list of "
                            "length *3* of ints or strings or tuples of ints "
                            "or strings")
        raise TypeError("{} must be a function that returns a list of "
                        "length *3* of floats or None")


def boundary_conditions(coords, volume, is_displacement_boundary,
                        is_force_boundary, is_tip):
    """Boundary-condition arrays and tips from the user's node functions
    (``peripy/model.py:1093-1212``).

    Each function is evaluated once per node; its per-component values
    (None: no condition) are gathered into arrays, and the arrays are
    formed with NumPy.  A force value is applied per unit volume of its
    node and shared equally among the nodes that carry any force condition.

    :returns: ``(bc_types, bc_values, force_bc_types, force_bc_values,
        tip_types, ntips)``; ``tip_types[tip]`` lists the ``(node,
        component)`` pairs of each tip in node, then component order
        (members of a tuple in their order) and ``ntips`` counts them, with
        ``ntips['model']`` the number of nodes.
    """
    funcs = (('is_displacement_boundary', is_displacement_boundary),
             ('is_force_boundary', is_force_boundary), ('is_tip', is_tip))
    for name, f in funcs:
        _check_node_function(name, f, coords[0][:])
    n = coords.shape[0]
    disp = np.zeros((n, 3))
    force = np.zeros((n, 3))
    bc_types = np.zeros((n, 3), dtype=np.intc)
    force_bc_types = np.zeros((n, 3), dtype=np.intc)
    tips = {}
    ntips = {'model': n}
    for i in range(n):
        x = coords[i][:]
        for j, v in enumerate(is_displacement_boundary(x)):
            if v is not None:
                disp[i, j] = v
                bc_types[i, j] = 1
        for j, v in enumerate(is_force_boundary(x)):
            if v is not None:
                force[i, j] = v
                force_bc_types[i, j] = 1
        for j, t in enumerate(is_tip(x)):
            if t is None:
                continue
            for name in (t if type(t) is tuple else (t,)):
                tips.setdefault(str(name), []).append((i, j))
    for name, entries in tips.items():
        ntips[name] = len(entries)
    bc_values = disp
    # per unit volume of the node, then shared among the force nodes
    force_bc_values = np.where(force_bc_types == 1,
                               force / volume[:, None], 0.0)
    force_nodes = int(np.count_nonzero(force_bc_types.any(axis=1)))
    if force_nodes:
        force_bc_values = force_bc_values / force_nodes
    return (bc_types, bc_values, force_bc_types, force_bc_values, tips,
            ntips)


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
        else:
            self.volume = _given_array("volume", volume, (self.nnodes,),
                                       np.float64, "(nnodes, )")

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
            self.family = _given_array("family", family, (self.nnodes,),
                                       np.intc, "(nnodes, )")
            nlist, n_neigh = _connectivity_pair(connectivity)
            warnings.warn("Reading connectivity from argument.")
            nlist = nlist.astype(np.intc)
            n_neigh = n_neigh.astype(np.intc)
            self.max_neighbours = np.intc(np.shape(nlist)[1])
            # the row width each integrator family works on: family.max()
            # for the CPU layout, a power of two for device integrators
            width = (1 << (int(self.family.max() - 1)).bit_length()
                     if integrator.context else self.family.max())
            fits = (self.max_neighbours & (self.max_neighbours - 1) == 0
                    if integrator.context
                    else self.max_neighbours == width)
            if not fits:
                raise ValueError(
                    "max_neighbours, which is equal to the size of axis 1 "
                    "of nlist is wrong (expected max_neighbours = "
                    "np.shape(nlist)[1] = {}, got {})".format(
                        width, self.max_neighbours))

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
        else:
            self.stiffness_corrections = _given_array(
                "stiffness_corrections", stiffness_corrections,
                (self.nnodes, self.max_neighbours), np.float64,
                "(nnodes, max_neighbours)")

        if is_bond_type is None:
            def is_bond_type(x, y):
                return 0

        (self.bond_stiffness, self.critical_stretch, self.plus_cs,
         self.nbond_types, self.nregimes) = damage_model(
             bond_stiffness, critical_stretch)

        if bond_types is None:
            self.bond_types = self._set_bond_types(
                self.initial_connectivity, is_bond_type, self.nbond_types,
                self.nregimes)
        else:
            self.bond_types = _given_array(
                "bond_types", bond_types, (self.nnodes, self.max_neighbours),
                np.intc, "(nnodes, max_neighbours)")

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
        """The damage model as :func:`damage_model` normalises it."""
        return damage_model(bond_stiffness, critical_stretch)

    def _set_boundary_conditions(self, is_displacement_boundary,
                                 is_force_boundary, is_tip):
        """BC arrays and tips (:func:`boundary_conditions`)."""
        return boundary_conditions(self.coords, self.volume,
                                   is_displacement_boundary,
                                   is_force_boundary, is_tip)

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
        displacement_bc_magnitudes = _schedule(
            "displacement_bc_magnitudes", displacement_bc_magnitudes,
            first_step, steps)
        force_bc_magnitudes = _schedule("force_bc_magnitudes",
                                        force_bc_magnitudes, first_step,
                                        steps)
        if connectivity is None:
            nlist, n_neigh = (a.copy() for a in self.initial_connectivity)
        else:
            nlist, n_neigh = _connectivity_pair(connectivity)
        shape = (self.nnodes, self.max_neighbours)
        if regimes is None:
            regimes = np.zeros(shape, dtype=np.intc)
        elif type(regimes) != np.ndarray:
            raise TypeError("regimes type is wrong (expected {} or {}, got "
                            "{})".format(np.ndarray, type(None),
                                         type(regimes)))
        elif np.shape(regimes) != shape:
            raise ValueError("regimes shape is wrong, and must be (nnodes, "
                             "max_neighbours) (expected {}, got {})".format(
                                 shape, np.shape(regimes)))
        else:
            regimes = regimes.astype(np.intc)
        if bond_stiffness is None and critical_stretch is None:
            (bond_stiffness, critical_stretch, plus_cs, nbond_types,
             nregimes) = (self.bond_stiffness, self.critical_stretch,
                          self.plus_cs, self.nbond_types, self.nregimes)
        else:
            (bond_stiffness, critical_stretch, plus_cs, nbond_types,
             nregimes) = damage_model(bond_stiffness, critical_stretch)
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
