"""ctypes binding of the C ABI declared in ``include/pp_gb300.h``.

The shared library ``libpp_gb300.so`` is built in-tree by
:mod:`probabilistic_peridynamics_gb300.build`.  There is no fallback: if the
library is missing or fails to load, :func:`lib` raises, so no caller can run
the step anywhere but on the CUDA kernels.
"""
import ctypes
import pathlib
import threading

_HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = _HERE / "libpp_gb300.so"

PP_SUCCESS = 0
PP_ERROR_INVALID_VALUE = 1
PP_ERROR_MAX_NEIGH = 2
PP_ERROR_MISALIGNED = 3
PP_ERROR_UNSUPPORTED = 4
PP_ERROR_CUDA = 5
PP_ERROR_TOO_LARGE = 6
PP_STATIC_MAX_STEPS = 65536

PP_EULER = 0
PP_EULER_CROMER = 1
PP_VELOCITY_VERLET = 2

PP_FLOAT64 = 0
PP_MIXED = 1

PP_FLAG_COMPENSATED = 1
PP_MIXED_VARIANTS = 3
PP_STATUS_OK = 0
PP_STATUS_COPY_TIMEOUT = 1
PP_STATUS_BAD_TILING = 2
PP_TILE_NODES_MAX = 128
PP_TILE_HALO_MAX = 768

_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_f64 = ctypes.c_double


class BondForceArgs(ctypes.Structure):
    """Mirror of ``pp_bond_force_args``."""

    _fields_ = [
        ("nnodes", _i32), ("max_neigh", _i32), ("nregimes", _i32),
        ("nbond_types", _i32),
        ("u", _vp), ("force", _vp), ("body_force", _vp), ("r0", _vp),
        ("vols", _vp), ("nlist", _vp), ("fc_types", _vp), ("fc_values", _vp),
        ("stiffness_corrections", _vp), ("bond_types", _vp),
        ("regimes", _vp), ("plus_cs", _vp), ("bond_stiffness_table", _vp),
        ("critical_stretch_table", _vp),
        ("bond_stiffness", _f64), ("critical_stretch", _f64),
        ("fc_scale", _f64),
    ]


class FusedArgs(ctypes.Structure):
    """Mirror of ``pp_fused_args``."""

    _fields_ = [
        ("nnodes", _i32), ("max_neigh", _i32), ("integrator", _i32),
        ("precision", _i32), ("nregimes", _i32), ("nbond_types", _i32),
        ("flags", _i32), ("nodes_per_block", _i32), ("variant", _i32),
        ("reserved", _i32),
        ("dt", _f64), ("damping", _f64), ("bond_stiffness", _f64),
        ("critical_stretch", _f64),
        ("bond_stiffness_table", _vp), ("critical_stretch_table", _vp),
        ("plus_cs", _vp),
        ("r0", _vp), ("vols", _vp), ("family", _vp), ("bc_types", _vp),
        ("bc_values", _vp), ("fc_types", _vp), ("fc_values", _vp),
        ("densities", _vp), ("stiffness_corrections", _vp),
        ("bond_types", _vp), ("bond_length", _vp), ("node_instance", _vp),
        ("instance_s0", _vp),
        ("ninstances", _i32), ("reserved2", _i32),
        ("nlist", _vp), ("regimes", _vp),
        ("u", _vp * 2), ("ud", _vp), ("udd", _vp), ("force", _vp),
        ("body_force", _vp), ("n_neigh", _vp), ("damage", _vp),
        ("rec", _vp * 2), ("ulo", _vp * 2), ("vel", _vp),
        ("acc", _vp), ("frc", _vp), ("rho32", _vp), ("sc32", _vp),
        ("nflags", _vp), ("umax", _vp), ("status", _vp),
        ("pos_scale", _f64), ("min_bond", _f64), ("pos_origin", _f64 * 3),
        ("tiling", _vp),
    ]


class Tiling(ctypes.Structure):
    """Mirror of ``pp_tiling``."""

    _fields_ = [
        ("ntiles", _i32), ("halo_cap", _i32),
        ("perm", _vp), ("inv", _vp), ("tile_start", _vp), ("halo", _vp),
        ("halo_count", _vp), ("own_off", _vp), ("tile_ref", _vp),
        ("row_off", _vp),
        ("entry", _vp), ("slot", _vp), ("bond_type", _vp), ("regime", _vp),
        ("correction", _vp), ("r0", _vp), ("bc_values", _vp),
        ("fc_values", _vp), ("node_instance", _vp), ("n_neigh", _vp),
        ("sched", _vp),
    ]


class CorrectionsArgs(ctypes.Structure):
    """Mirror of ``pp_corrections_args``."""
    _fields_ = [
        ("nnodes", _i32), ("max_neigh", _i32),
        ("micromodulus_function", _i32), ("volume_correction", _i32),
        ("surface_correction", _i32), ("reserved", _i32),
        ("micromodulus_horizon", _f64), ("vc_horizon", _f64),
        ("vc_node_radius", _f64), ("family_volume_bulk", _f64),
        ("average_volume", _f64),
        ("r0", _vp), ("volume", _vp), ("nlist", _vp), ("n_neigh", _vp),
        ("corrections", _vp), ("family_volume", _vp),
    ]


class WriteSumsArgs(ctypes.Structure):
    """Mirror of ``pp_write_sums_args``."""
    _fields_ = [
        ("nnodes", _i32), ("ntips", _i32), ("leaves3", _i32),
        ("values3", _i32), ("leaves1", _i32), ("values1", _i32),
        ("u", _vp), ("ud", _vp), ("udd", _vp), ("force", _vp),
        ("body_force", _vp), ("damage", _vp), ("volume", _vp),
        ("plan3", _vp), ("plan1", _vp), ("tip_offsets", _vp),
        ("tip_entries", _vp), ("scratch", _vp), ("sums", _vp),
    ]


class AdjointArgs(ctypes.Structure):
    """Mirror of ``pp_adjoint_args``."""

    _fields_ = [
        ("nnodes", _i32), ("max_neigh", _i32), ("dt", _f64),
        ("r0", _vp), ("vols", _vp), ("nlist", _vp), ("partner", _vp),
        ("bc_types", _vp), ("stiffness", _vp),
    ]


#: Every symbol the header declares, with (restype, argtypes).
SIGNATURES = {
    "pp_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "pp_abi_version": (ctypes.c_int, []),
    "pp_bond_force": (ctypes.c_int, [ctypes.POINTER(BondForceArgs), _vp]),
    "pp_damage": (ctypes.c_int, [_vp, _vp, _vp, _vp, _i32, _i32, _vp]),
    "pp_update_displacement_euler": (
        ctypes.c_int, [_vp, _vp, _vp, _vp, _f64, _f64, _i64, _vp]),
    "pp_update_displacement_euler_cromer": (
        ctypes.c_int,
        [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _f64, _f64, _f64, _i64, _vp]),
    "pp_update_displacement_velocity_verlet": (
        ctypes.c_int,
        [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _f64, _f64, _f64, _i64, _vp]),
    "pp_fused_step": (
        ctypes.c_int, [ctypes.POINTER(FusedArgs), _i32, _f64, _f64, _vp]),
    "pp_fused_run": (
        ctypes.c_int,
        [ctypes.POINTER(FusedArgs), _i32, _i64, _vp, _vp, _i64, _i32, _i32,
         _vp, _vp]),
    "pp_bond_extent": (ctypes.c_int, [_vp, _vp, _i32, _i32, _vp, _vp]),
    "pp_stiffness_corrections": (ctypes.c_int,
                                 [ctypes.POINTER(CorrectionsArgs), _vp]),
    "pp_neighbour_cells": (ctypes.c_int, [_vp, _i32, _vp, _f64, _vp, _vp, _vp,
                                          _vp]),
    "pp_neighbour_rows": (ctypes.c_int, [_vp, _i32, _f64, _vp, _f64, _vp, _vp,
                                         _vp, _i32, _vp, _vp, _vp, _vp]),
    "pp_create_crack": (ctypes.c_int, [_vp, _i32, _i32, _i32, _vp, _vp, _vp,
                                       _vp, _vp]),
    "pp_pairwise_plan": (ctypes.c_int64, [_i64, _vp, _i64]),
    "pp_bond_lengths": (ctypes.c_int, [_vp, _vp, _i32, _i32, _vp, _vp]),
    "pp_cy_break_bonds": (ctypes.c_int, [_vp, _vp, _vp, _vp, _i32, _i32,
                                         _f64, _vp]),
    "pp_cy_bond_force": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _f64, _vp,
                                        _vp, _f64, _i32, _i32, _vp, _vp]),
    "pp_cy_break_and_force": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _f64,
                                             _f64, _vp, _vp, _f64, _i32,
                                             _i32, _vp, _vp, _vp]),
    "pp_cy_update_displacement": (ctypes.c_int, [_vp, _vp, _vp, _vp, _f64,
                                                 _f64, _i32, _vp]),
    "pp_cy_damage": (ctypes.c_int, [_vp, _vp, _i32, _vp, _vp]),
    "pp_write_sums": (ctypes.c_int, [ctypes.POINTER(WriteSumsArgs), _vp]),
    "pp_mixed_pack": (ctypes.c_int, [ctypes.POINTER(FusedArgs), _i32, _vp]),
    "pp_mixed_export": (ctypes.c_int, [ctypes.POINTER(FusedArgs), _i32, _vp]),
    "pp_partner_slots": (ctypes.c_int, [_vp, _i32, _i32, _vp, _vp]),
    "pp_mark_breaks": (ctypes.c_int, [_vp, _vp, _i64, _i32, _vp]),
    "pp_bonds_at_step": (ctypes.c_int, [_vp, _vp, _i64, _i32, _vp, _vp]),
    "pp_adjoint_backward": (
        ctypes.c_int, [ctypes.POINTER(AdjointArgs), _vp, _vp, _vp, _vp, _vp]),
    "pp_fused_run_static": (
        ctypes.c_int, [ctypes.POINTER(FusedArgs), _i32, _i64, _vp, _vp, _vp]),
    "pp_static_status": (ctypes.c_int, [_vp, _vp]),
    "pp_cy_check_symmetric": (ctypes.c_int, [_vp, _vp, _i32, _i32, _vp,
                                             _vp]),
    "pp_tile_halos": (ctypes.c_int, [ctypes.POINTER(FusedArgs),
                                     ctypes.POINTER(Tiling), _vp]),
    "pp_tile_rows": (ctypes.c_int, [ctypes.POINTER(FusedArgs),
                                    ctypes.POINTER(Tiling), _vp]),
    "pp_host_register": (ctypes.c_int, [_vp, ctypes.c_size_t]),
    "pp_host_unregister": (ctypes.c_int, [_vp]),
}

_lock = threading.Lock()
_lib = None


class LibraryError(RuntimeError):
    """The CUDA library is missing, failed to load or returned an error."""


def lib():
    """Load ``libpp_gb300.so`` once and return the ctypes handle."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise LibraryError(
                    f"{LIB_PATH} is missing; build it with "
                    "`python -m probabilistic_peridynamics_gb300.build`")
            handle = ctypes.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
        return _lib


def check(status, what):
    """Raise :class:`LibraryError` for a non-zero status code."""
    if status != PP_SUCCESS:
        text = lib().pp_status_string(status).decode()
        raise LibraryError(f"{what} failed: {text} (status {status})")
