"""Many independent models stepped together (outer-loop uncertainty
quantification).

PeriPy runs one model per ``Model.simulate`` call.  For Monte-Carlo studies
over material parameters the same time step is run for many samples; here
the samples ("instances") are concatenated into one node set -- bonds never
cross instances -- and advanced by one persistent fused kernel per step,
with the runs of steps captured in a CUDA graph (``pp_fused_run``) and the
kernel's tile shape picked by the autotuner.  Each node carries its
instance index; the per-instance critical stretch comes from a small table
(``pp_fused_args.node_instance`` / ``instance_s0``), and per-bond stiffness
noise enters as ``stiffness_corrections`` (``peripy/cl/peridynamics.cl:214``
semantics).
"""
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Instance:
    """One sample: the arrays ``Integrator.build``/``create_buffers`` take
    for a single model, plus its critical stretch."""

    coords: np.ndarray
    volume: np.ndarray
    family: np.ndarray
    nlist: np.ndarray
    n_neigh: np.ndarray
    bc_types: np.ndarray
    bc_values: np.ndarray
    critical_stretch: float
    force_bc_types: np.ndarray = None
    force_bc_values: np.ndarray = None
    densities: np.ndarray = None
    stiffness_corrections: np.ndarray = None
    meta: dict = field(default_factory=dict)

    @property
    def nnodes(self):
        return self.coords.shape[0]


def pair_noise(nlist, lo, hi, seed):
    """Per-slot factors uniform in [lo, hi), equal for the two directions of
    each bond: a hash (splitmix64) of the unordered node pair and ``seed``.

    Padding and broken slots (-1) get 1.0.
    """
    n = nlist.shape[0]
    i = np.broadcast_to(np.arange(n, dtype=np.uint64)[:, None], nlist.shape)
    valid = nlist >= 0
    j = np.where(valid, nlist, 0).astype(np.uint64)
    a = np.minimum(i, j)
    b = np.maximum(i, j)
    with np.errstate(over="ignore"):
        z = (a << np.uint64(32)) | b
        z = z ^ np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))
    return np.where(valid, lo + (hi - lo) * u, 1.0)


@dataclass
class Batch:
    """Instances concatenated into one model (global node indices)."""

    instances: list
    offsets: np.ndarray          # node offset of each instance, len + 1
    max_neigh: int
    coords: np.ndarray
    volume: np.ndarray
    family: np.ndarray
    nlist: np.ndarray
    n_neigh: np.ndarray
    bc_types: np.ndarray
    bc_values: np.ndarray
    force_bc_types: np.ndarray
    force_bc_values: np.ndarray
    densities: np.ndarray
    stiffness_corrections: np.ndarray
    node_instance: np.ndarray
    instance_s0: np.ndarray

    @property
    def nnodes(self):
        return self.coords.shape[0]

    @property
    def bonds(self):
        return int(self.family.sum())

    def split(self, array, kind="node"):
        """Per-instance views of a concatenated node array, or of a
        concatenated neighbour list mapped back to local indices."""
        out = []
        for k in range(len(self.instances)):
            a, b = self.offsets[k], self.offsets[k + 1]
            part = array[a:b]
            if kind == "nlist":
                w = self.instances[k].nlist.shape[1]
                part = np.where(part[:, :w] >= 0, part[:, :w] - a, -1)
            out.append(part)
        return out


def concatenate(instances):
    """Concatenate instances; rows are padded to the widest neighbour list."""
    if not instances:
        raise ValueError("no instances")
    if len(instances) > 256:
        raise ValueError("at most 256 instances per batch (got {})".format(
            len(instances)))
    width = max(inst.nlist.shape[1] for inst in instances)
    sizes = np.array([inst.nnodes for inst in instances])
    offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    n = int(offsets[-1])
    nlist = np.full((n, width), -1, dtype=np.intc)
    corr = np.ones((n, width))
    any_corr = any(inst.stiffness_corrections is not None
                   for inst in instances)
    dyn = [inst.densities is not None for inst in instances]
    if any(dyn) and not all(dyn):
        raise ValueError("densities must be given for all instances or none")

    def cat(name, default_shape, dtype):
        parts = []
        for inst in instances:
            v = getattr(inst, name)
            parts.append(np.zeros((inst.nnodes,) + default_shape, dtype=dtype)
                         if v is None else np.asarray(v, dtype=dtype))
        return np.concatenate(parts)

    for k, inst in enumerate(instances):
        a, b = offsets[k], offsets[k + 1]
        w = inst.nlist.shape[1]
        nl = inst.nlist
        nlist[a:b, :w] = np.where(nl >= 0, nl + a, -1)
        if inst.stiffness_corrections is not None:
            corr[a:b, :w] = inst.stiffness_corrections
    return Batch(
        instances=list(instances), offsets=offsets, max_neigh=int(width),
        coords=cat("coords", (3,), np.float64),
        volume=cat("volume", (), np.float64),
        family=cat("family", (), np.intc), nlist=nlist,
        n_neigh=cat("n_neigh", (), np.intc),
        bc_types=cat("bc_types", (3,), np.intc),
        bc_values=cat("bc_values", (3,), np.float64),
        force_bc_types=cat("force_bc_types", (3,), np.intc),
        force_bc_values=cat("force_bc_values", (3,), np.float64),
        densities=cat("densities", (3,), np.float64) if all(dyn) else None,
        stiffness_corrections=corr if any_corr else None,
        node_instance=np.repeat(np.arange(len(instances), dtype=np.intc),
                                sizes),
        instance_s0=np.array([inst.critical_stretch for inst in instances],
                             dtype=np.float64))


class BatchedSimulation:
    """Steps a :class:`Batch` with one CUDA integrator.

    :arg batch: the concatenated instances.
    :arg integrator: a fused CUDA integrator (``EulerCUDA``,
        ``EulerCromerCUDA``, ``VelocityVerletCUDA``), not yet built.
    :arg float bond_stiffness: the micro-modulus shared by all instances
        (per-instance and per-bond variation goes into the stiffness
        corrections).
    """

    def __init__(self, batch, integrator, bond_stiffness):
        if not integrator.fused:
            raise ValueError("batched instances need a fused integrator")
        self.batch = batch
        self.integrator = integrator
        self.bond_stiffness = float(bond_stiffness)
        integrator.set_instances(batch.node_instance, batch.instance_s0)
        integrator.build(batch.nnodes, 3, batch.max_neigh, batch.coords,
                         batch.volume, batch.family, batch.bc_types,
                         batch.bc_values, batch.force_bc_types,
                         batch.force_bc_values, batch.stiffness_corrections,
                         None, batch.densities)
        self.reset()

    def reset(self):
        """(Re)load the initial state: zero displacement and velocity."""
        b = self.batch
        z = np.zeros((b.nnodes, 3))
        self.integrator.create_buffers(
            b.nlist, b.n_neigh, self.bond_stiffness,
            float(b.instance_s0[0]), None, z, z, z, z, z,
            np.zeros(b.nnodes), None, 1, 1)
        self.step = 0

    def run(self, steps, displacement_bc_magnitudes, force_bc_magnitudes=None):
        """Advance all instances by ``steps`` steps (magnitudes indexed from
        the current step)."""
        if force_bc_magnitudes is None:
            force_bc_magnitudes = np.zeros(len(displacement_bc_magnitudes))
        self.integrator._run(displacement_bc_magnitudes, force_bc_magnitudes,
                             self.step, steps)
        self.step += steps

    def results(self):
        """Per-instance ``(u, ud, damage, nlist, n_neigh)``."""
        b = self.batch
        z = lambda: np.zeros((b.nnodes, 3))  # noqa: E731
        (u, ud, udd, force, body, damage, nlist,
         n_neigh) = self.integrator.write(
             z(), z(), z(), z(), z(), np.zeros(b.nnodes), b.nlist.copy(),
             b.n_neigh.copy())
        return list(zip(b.split(u), b.split(ud), b.split(damage),
                        b.split(nlist, "nlist"), b.split(n_neigh)))


def uq_instances(count=64, seed=2024, nx_range=(60, 200), ny_range=(60, 200),
                 nz=5, dx=0.005, s0_mean=0.005, s0_sigma=0.2, noise=(0.9, 1.1),
                 density=2400.0):
    """The batched UQ workload: ``count`` plates nx x ny x nz (nx, ny drawn
    uniformly), critical stretch lognormal with the given mean and sigma of
    the underlying normal, per-bond stiffness noise uniform in ``noise``
    (symmetric per bond pair), x faces pulled apart, densities ``density``.
    """
    from .lattice import face_bcs, lattice_coords, lattice_family
    rng = np.random.default_rng(seed)
    mu = np.log(s0_mean) - s0_sigma ** 2 / 2
    out = []
    for k in range(count):
        nx = int(rng.integers(nx_range[0], nx_range[1] + 1))
        ny = int(rng.integers(ny_range[0], ny_range[1] + 1))
        coords = lattice_coords(nx, ny, nz, dx)
        family, nlist, _ = lattice_family(nx, ny, nz, 3.015)
        bc_types, bc_values = face_bcs(coords, 0)
        n = coords.shape[0]
        out.append(Instance(
            coords=coords, volume=np.full(n, dx ** 3), family=family,
            nlist=nlist, n_neigh=family.copy(), bc_types=bc_types,
            bc_values=bc_values,
            critical_stretch=float(rng.lognormal(mu, s0_sigma)),
            densities=np.full((n, 3), density),
            stiffness_corrections=pair_noise(nlist, noise[0], noise[1],
                                             seed * 1000003 + k),
            meta={"nx": nx, "ny": ny, "nz": nz}))
    return out
