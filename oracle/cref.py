"""ctypes loader of ``oracle/pp_oracle.c`` (TEST INFRASTRUCTURE).

:func:`build` compiles the C restatement with ``-O2 -ffp-contract=off
-fopenmp`` into ``oracle/libpp_oracle.so`` (git-ignored, rebuilt on each
machine).  :class:`Stepper` has the interface of
:class:`oracle.cl_step.Stepper` and is bit-identical to it.
"""
import ctypes
import os
import pathlib
import subprocess

import numpy as np

from . import cl_step

HERE = pathlib.Path(__file__).resolve().parent
SRC = HERE / "pp_oracle.c"
LIB = HERE / "libpp_oracle.so"
_lib = None


def build(quiet=True):
    if LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cc = os.environ.get("CC", "gcc")
    cmd = [cc, "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-fPIC", "-shared", str(SRC), "-o", str(LIB) + ".tmp", "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    os.replace(str(LIB) + ".tmp", LIB)
    if not quiet:
        print("built", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(str(LIB))
        vp, i32, i64, f64 = (ctypes.c_void_p, ctypes.c_int, ctypes.c_int64,
                             ctypes.c_double)
        _lib.pp_oracle_bond_force.restype = ctypes.c_int
        _lib.pp_oracle_bond_force.argtypes = [
            i32, i32, vp, vp, vp, vp, vp, vp, f64, f64, f64, vp, vp, vp, vp,
            vp, vp, i32, vp, vp]
        _lib.pp_oracle_damage.restype = None
        _lib.pp_oracle_damage.argtypes = [i32, i32, vp, vp, vp, vp]
        _lib.pp_oracle_update.restype = None
        _lib.pp_oracle_update.argtypes = [i32, i64, vp, vp, vp, vp, vp, vp,
                                          vp, f64, f64, f64]
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dtype):
    return None if a is None else np.ascontiguousarray(a, dtype=dtype)


_KIND = {"euler": 0, "euler_cromer": 1, "velocity_verlet": 2}


class Stepper(cl_step.Stepper):
    """C-backed :class:`oracle.cl_step.Stepper` (same results, faster)."""

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        n = self.r0.shape[0]
        self.r0 = _c(self.r0, np.float64)
        self.vols = _c(self.vols, np.float64)
        self.fc_types = _c(self.fc_types, np.intc)
        self.fc_values = _c(self.fc_values, np.float64)
        self.bc_types = _c(self.bc_types, np.intc)
        self.bc_values = _c(self.bc_values, np.float64)
        self.densities = (np.ones((n, 3)) if self.densities is None
                          else _c(self.densities, np.float64))
        self.sc = _c(self.sc, np.float64)
        self.bond_types = _c(self.bond_types, np.intc)
        if self.bond_types is not None:
            self.k_tab = _c(np.asarray(self.k).ravel(), np.float64)
            self.s_tab = _c(np.asarray(self.s0).ravel(), np.float64)
            self.c_tab = _c(np.asarray(self.plus_cs).ravel(), np.float64)
            self.k_s = self.s_s = 0.0
        else:
            self.k_tab = self.s_tab = self.c_tab = None
            self.k_s, self.s_s = float(self.k), float(self.s0)

    def step(self, displacement_bc_magnitude, force_bc_magnitude):
        L = lib()
        n, mn = self.nlist.shape
        rc = L.pp_oracle_bond_force(
            n, mn, _p(self.u), _p(self.r0), _p(self.vols), _p(self.nlist),
            _p(self.fc_types), _p(self.fc_values), float(force_bc_magnitude),
            self.k_s, self.s_s, _p(self.sc), _p(self.bond_types),
            _p(self.regimes), _p(self.k_tab), _p(self.s_tab),
            _p(self.c_tab), int(self.nregimes), _p(self.force),
            _p(self.body_force))
        if rc != 0:
            raise ValueError("max_neigh must be a power of two <= 1024")
        L.pp_oracle_update(
            _KIND[self.integrator], 3 * n, _p(self.force), _p(self.u),
            _p(self.ud), _p(self.udd), _p(self.bc_types), _p(self.bc_values),
            _p(self.densities), float(displacement_bc_magnitude),
            float(self.damping), float(self.dt))

    def write(self):
        n, mn = self.nlist.shape
        n_neigh = np.zeros(n, dtype=np.intc)
        dmg = np.zeros(n)
        fam = _c(self.family, np.intc)
        lib().pp_oracle_damage(n, mn, _p(self.nlist), _p(fam), _p(n_neigh),
                               _p(dmg))
        return (self.u.copy(), self.ud.copy(), self.udd.copy(),
                self.force.copy(), self.body_force.copy(), dmg,
                self.nlist.copy(), n_neigh)
