"""C-ABI library checks that need no GPU.

* ``libpp_gb300.so`` loads and exports every function ``include/pp_gb300.h``
  declares, with the ctypes mirror structs sized like the C structs;
* argument validation runs on the host, before any CUDA call, and returns
  the documented status codes;
* the fixed-point position frame is exact for neighbour differences.
"""
import ctypes
import pathlib
import re

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "pp_gb300.h"


@pytest.fixture(scope="module")
def L():
    from probabilistic_peridynamics_gb300 import _lib
    if not _lib.LIB_PATH.exists():
        from probabilistic_peridynamics_gb300 import build
        build.build()
    return _lib.lib()


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pp_[a-z0-9_]+)\s*\(", text)))


def test_header_functions_exported(L):
    from probabilistic_peridynamics_gb300 import _lib
    names = declared_functions()
    assert names, "no declarations parsed"
    for name in names:
        assert hasattr(L, name), f"{name} not exported"
    assert set(names) == set(_lib.SIGNATURES), (
        "ctypes signatures out of sync with the header")


def test_abi_version_and_status_strings(L):
    assert L.pp_abi_version() == 3
    assert L.pp_status_string(0) == b"success"
    assert b"power of two" in L.pp_status_string(2)


def test_struct_layout_matches_header():
    """Field order and sizes of the ctypes mirrors (LP64 C layout)."""
    from probabilistic_peridynamics_gb300 import _lib
    # pp_bond_force_args: 4 int32, 14 pointers, 3 doubles
    assert ctypes.sizeof(_lib.BondForceArgs) == 4 * 4 + 14 * 8 + 3 * 8
    # pp_fused_args: 10 int32 then doubles and pointers
    f = dict((n, getattr(_lib.FusedArgs, n)) for n, _ in
             _lib.FusedArgs._fields_)
    assert f["variant"].offset == 32
    assert f["dt"].offset == 40
    assert f["bond_stiffness_table"].offset == 72
    assert f["bond_length"].offset == f["bond_types"].offset + 8
    assert f["pos_origin"].offset + 24 == f["tiling"].offset
    assert f["tiling"].offset + 8 == ctypes.sizeof(_lib.FusedArgs)
    # pp_tiling: 2 int32 then 19 pointers
    assert ctypes.sizeof(_lib.Tiling) == 2 * 4 + 19 * 8
    assert _lib.Tiling.perm.offset == 8
    assert _lib.Tiling.sched.offset == 8 + 18 * 8


def test_struct_layout_matches_c_compiler(tmp_path):
    """sizeof and offsetof of the C structs, compiled from the header with
    the host C compiler, equal the ctypes mirrors."""
    import shutil
    import subprocess
    from probabilistic_peridynamics_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    checks = {"pp_fused_args": (_lib.FusedArgs, ("variant", "dt", "nlist",
                                                "rec", "pos_origin",
                                                "tiling")),
              "pp_tiling": (_lib.Tiling, ("perm", "tile_ref", "entry",
                                          "correction", "n_neigh", "sched")),
              "pp_corrections_args": (_lib.CorrectionsArgs, ("r0",)),
              "pp_write_sums_args": (_lib.WriteSumsArgs, ("u", "sums")),
              "pp_adjoint_args": (_lib.AdjointArgs, ("r0", "stiffness"))}
    lines = ['#include <stdio.h>', '#include <stddef.h>',
             f'#include "{HEADER}"', "int main(void) {"]
    for struct, (_, fields) in checks.items():
        lines.append(f'printf("{struct} %zu\\n", sizeof({struct}));')
        for f in fields:
            lines.append(f'printf("{struct}.{f} %zu\\n", '
                         f'offsetof({struct}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run(
        [str(exe)], check=True, capture_output=True,
        text=True).stdout.splitlines())
    for struct, (cls, fields) in checks.items():
        assert int(out[struct]) == ctypes.sizeof(cls), struct
        for f in fields:
            assert int(out[f"{struct}.{f}"]) == getattr(cls, f).offset, f
    # pp_corrections_args: 6 int32, 5 doubles, 6 pointers
    assert ctypes.sizeof(_lib.CorrectionsArgs) == 6 * 4 + 5 * 8 + 6 * 8
    assert _lib.CorrectionsArgs.r0.offset == 64


def test_validation_without_gpu(L):
    from probabilistic_peridynamics_gb300 import _lib
    a = _lib.BondForceArgs()
    a.nnodes, a.max_neigh = 10, 3
    assert L.pp_bond_force(ctypes.byref(a), None) == _lib.PP_ERROR_MAX_NEIGH
    a.max_neigh = 2048
    assert L.pp_bond_force(ctypes.byref(a), None) == _lib.PP_ERROR_MAX_NEIGH
    a.max_neigh = 4
    # NULL pointers with nnodes > 0
    assert L.pp_bond_force(ctypes.byref(a), None) == \
        _lib.PP_ERROR_INVALID_VALUE
    assert L.pp_bond_force(None, None) == _lib.PP_ERROR_INVALID_VALUE
    a.nnodes = 0
    assert L.pp_bond_force(ctypes.byref(a), None) == _lib.PP_SUCCESS
    assert L.pp_damage(None, None, None, None, 5, 6, None) == \
        _lib.PP_ERROR_MAX_NEIGH
    assert L.pp_update_displacement_euler(None, None, None, None, 0.0, 1.0,
                                          -1, None) == \
        _lib.PP_ERROR_INVALID_VALUE
    fa = _lib.FusedArgs()
    fa.nnodes, fa.max_neigh = 4, 4
    assert L.pp_fused_step(ctypes.byref(fa), 2, 0.0, 0.0, None) == \
        _lib.PP_ERROR_INVALID_VALUE
    fa.integrator = 7
    assert L.pp_fused_step(ctypes.byref(fa), 0, 0.0, 0.0, None) == \
        _lib.PP_ERROR_INVALID_VALUE
    fa.integrator = 0
    fa.precision = 9
    assert L.pp_fused_step(ctypes.byref(fa), 0, 0.0, 0.0, None) == \
        _lib.PP_ERROR_INVALID_VALUE
    # flags: unknown bits, and compensation outside PP_MIXED
    fa.precision = _lib.PP_FLOAT64
    fa.flags = 2
    assert L.pp_fused_step(ctypes.byref(fa), 0, 0.0, 0.0, None) == \
        _lib.PP_ERROR_INVALID_VALUE
    fa.flags = _lib.PP_FLAG_COMPENSATED
    assert L.pp_fused_step(ctypes.byref(fa), 0, 0.0, 0.0, None) == \
        _lib.PP_ERROR_UNSUPPORTED
    fa.flags = 0
    # misaligned mixed-precision pointers are rejected before any launch
    buf = (ctypes.c_char * 64)()
    base = ctypes.addressof(buf)
    for name in ("r0", "vols", "family", "bc_types", "bc_values",
                 "fc_types", "fc_values", "nlist", "n_neigh", "frc",
                 "nflags", "umax", "status"):
        setattr(fa, name, base)
    fa.precision = _lib.PP_MIXED
    fa.rec[0] = base + 16  # records must be 32-byte aligned
    fa.rec[1] = base
    fa.ulo[0] = fa.ulo[1] = base
    fa.pos_scale = 1.0
    assert L.pp_fused_step(ctypes.byref(fa), 0, 0.0, 0.0, None) == \
        _lib.PP_ERROR_MISALIGNED


def test_bond_lengths_validation_without_gpu(L):
    from probabilistic_peridynamics_gb300 import _lib
    assert L.pp_bond_lengths(None, None, 10, 2000, None, None) == \
        _lib.PP_ERROR_MAX_NEIGH
    assert L.pp_bond_lengths(None, None, 10, 0, None, None) == \
        _lib.PP_ERROR_MAX_NEIGH
    assert L.pp_bond_lengths(None, None, 0, 4, None, None) == _lib.PP_SUCCESS
    assert L.pp_bond_lengths(None, None, 10, 4, None, None) == \
        _lib.PP_ERROR_INVALID_VALUE
    assert L.pp_bond_lengths(None, None, -1, 4, None, None) == \
        _lib.PP_ERROR_INVALID_VALUE


def test_fixed_point_frame_exact_differences():
    from probabilistic_peridynamics_gb300.integrators import _pos_frame
    rng = np.random.default_rng(0)
    coords = rng.uniform(-3.0, 5.0, size=(1000, 3))
    extent = 0.3
    origin, step = _pos_frame(coords, extent)
    assert np.log2(step) == int(np.log2(step))  # a power of two
    assert extent / step <= 2 ** 21
    q = np.rint((coords - origin) / step)
    assert np.all(np.abs(q) < 2 ** 30)
    assert np.all(np.abs(origin + q * step - coords) <= step / 2)
    # bonds no longer than the extent give |dq| < 2**22: exact in float
    dq = np.abs(q[1:] - q[:-1])
    short = np.all(np.abs(coords[1:] - coords[:-1]) <= extent, axis=1)
    assert np.all(dq[short] < 2 ** 22)


def test_magic_conversion_exact():
    """float(q) = bits(0x4B400000 + q) - 1.5*2**23 for |q| < 2**22."""
    q = np.array([-(2 ** 22) + 1, -12345, -1, 0, 1, 777, 2 ** 22 - 1],
                 dtype=np.int32)
    bits = (q + np.int32(0x4B400000)).astype(np.int32)
    f = bits.view(np.float32).astype(np.float64) - 12582912.0
    assert np.array_equal(f, q.astype(np.float64))
