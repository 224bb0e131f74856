"""Minimal legacy-VTK mesh reader and writer, and a Gmsh MSH 2.x reader.

PeriPy reads meshes with meshio (``peripy/model.py:481-503``) and writes
them with ``meshio.write_points_cells`` (``peripy/model.py:505-534``).
meshio is not a dependency here, so this module reads and writes the subset
of the legacy VTK format those calls use: ``DATASET UNSTRUCTURED_GRID`` with
``POINTS``, ``CELLS`` and ``CELL_TYPES`` sections, ASCII or BINARY
(big-endian), version 4.x layout, plus ``POINT_DATA`` on write.
"""
from collections import namedtuple
import pathlib

import numpy as np

#: VTK cell-type ids and their names (the names meshio uses in cells_dict).
VTK_CELL_NAMES = {1: "vertex", 3: "line", 5: "triangle", 9: "quad",
                  10: "tetra", 12: "hexahedron"}
_VTK_CELL_IDS = {v: k for k, v in VTK_CELL_NAMES.items()}

_VTK_DTYPES = {"float": ">f4", "double": ">f8", "int": ">i4",
               "unsigned_int": ">u4", "long": ">i8", "vtkidtype": ">i4"}

Mesh = namedtuple("Mesh", ["points", "cells_dict"])


class MeshFormatError(ValueError):
    """The file is not a legacy VTK unstructured grid this reader handles."""


def _read_block(buf, pos, count, dtype, binary):
    """Read ``count`` values starting at byte ``pos``; return (array, pos)."""
    if binary:
        dt = np.dtype(_VTK_DTYPES[dtype])
        # The binary block starts after the header line's newline.
        nbytes = count * dt.itemsize
        arr = np.frombuffer(buf, dtype=dt, count=count, offset=pos)
        pos += nbytes
        # Skip the newline that terminates the binary block.
        while pos < len(buf) and buf[pos:pos + 1] in (b"\n", b"\r"):
            pos += 1
        return arr.astype(dt.newbyteorder("=")), pos
    values = []
    while len(values) < count:
        end = buf.index(b"\n", pos)
        values.extend(buf[pos:end].split())
        pos = end + 1
    kind = float if dtype in ("float", "double") else int
    return np.array([kind(v) for v in values[:count]]), pos


def _next_line(buf, pos):
    end = buf.find(b"\n", pos)
    if end < 0:
        end = len(buf)
    return buf[pos:end].decode("ascii", "replace").strip(), end + 1


def read_vtk(filename):
    """Read a legacy VTK unstructured grid.

    :returns: :class:`Mesh` with ``points`` (n, 3) float64 and
        ``cells_dict`` mapping a cell name ("triangle", "tetra", "line", ...)
        to an (ncells, nverts) int array.
    """
    buf = pathlib.Path(filename).read_bytes()
    pos = 0
    header, pos = _next_line(buf, pos)
    if not header.startswith("# vtk DataFile"):
        raise MeshFormatError(f"{filename}: not a legacy VTK file")
    _, pos = _next_line(buf, pos)  # title
    fmt, pos = _next_line(buf, pos)
    binary = fmt.upper() == "BINARY"
    points = None
    cells = None
    cell_types = None
    while pos < len(buf):
        line, pos = _next_line(buf, pos)
        if not line:
            continue
        words = line.split()
        key = words[0].upper()
        if key == "DATASET":
            if words[1].upper() != "UNSTRUCTURED_GRID":
                raise MeshFormatError(f"unsupported dataset {words[1]}")
        elif key == "POINTS":
            n = int(words[1])
            arr, pos = _read_block(buf, pos, 3 * n, words[2].lower(), binary)
            points = arr.reshape(n, 3).astype(np.float64)
        elif key == "CELLS":
            size = int(words[2])
            cells, pos = _read_block(buf, pos, size, "int", binary)
        elif key == "CELL_TYPES":
            n = int(words[1])
            cell_types, pos = _read_block(buf, pos, n, "int", binary)
        elif key in ("POINT_DATA", "CELL_DATA", "METADATA", "FIELD"):
            break
        else:
            raise MeshFormatError(f"unsupported VTK section {words[0]}")
    if points is None:
        raise MeshFormatError(f"{filename}: no POINTS section")
    cells_dict = {}
    if cells is not None and cell_types is not None:
        groups = {}
        p = 0
        for ctype in cell_types:
            npts = int(cells[p])
            groups.setdefault(int(ctype), []).append(cells[p + 1:p + 1 + npts])
            p += npts + 1
        for ctype, rows in groups.items():
            name = VTK_CELL_NAMES.get(ctype, str(ctype))
            cells_dict[name] = np.array(rows, dtype=np.int64)
    return Mesh(points, cells_dict)


def write_vtk(filename, points, cells=(), point_data=None, binary=True):
    """Write a legacy VTK 4.2 unstructured grid.

    :arg cells: sequence of ``(name, (ncells, nverts) array)`` pairs.
    :arg dict point_data: name -> (n,) or (n, k) array; ``None`` values are
        skipped (as meshio does for the ``damage``/``displacements`` fields).
    """
    points = np.asarray(points, dtype=np.float64)
    n = points.shape[0]
    out = bytearray()

    def put_line(text):
        out.extend(text.encode("ascii") + b"\n")

    def put_values(arr, dtype):
        arr = np.asarray(arr)
        if binary:
            out.extend(arr.astype(_VTK_DTYPES[dtype]).tobytes())
            out.extend(b"\n")
        else:
            put_line(" ".join(repr(v) for v in arr.ravel().tolist()))

    put_line("# vtk DataFile Version 4.2")
    put_line("written by probabilistic_peridynamics_gb300")
    put_line("BINARY" if binary else "ASCII")
    put_line("DATASET UNSTRUCTURED_GRID")
    put_line(f"POINTS {n} double")
    put_values(points.ravel(), "double")
    cells = [(name, np.asarray(c, dtype=np.int64)) for name, c in cells]
    ncells = sum(c.shape[0] for _, c in cells)
    if ncells:
        size = sum(c.shape[0] * (c.shape[1] + 1) for _, c in cells)
        put_line(f"CELLS {ncells} {size}")
        flat = np.concatenate([
            np.hstack([np.full((c.shape[0], 1), c.shape[1]), c]).ravel()
            for _, c in cells])
        put_values(flat, "int")
        put_line(f"CELL_TYPES {ncells}")
        types = np.concatenate([np.full(c.shape[0], _VTK_CELL_IDS[name])
                                for name, c in cells])
        put_values(types, "int")
    fields = {k: v for k, v in (point_data or {}).items() if v is not None}
    if fields:
        put_line(f"POINT_DATA {n}")
        put_line(f"FIELD FieldData {len(fields)}")
        for name, arr in fields.items():
            arr = np.asarray(arr, dtype=np.float64).reshape(n, -1)
            put_line(f"{name} {arr.shape[1]} {n} double")
            put_values(arr.ravel(), "double")
    pathlib.Path(filename).write_bytes(bytes(out))


#: Gmsh element types (MSH 2) and their node counts, named as meshio names
#: them in cells_dict.
MSH_ELEMENTS = {1: ("line", 2), 2: ("triangle", 3), 3: ("quad", 4),
                4: ("tetra", 4), 5: ("hexahedron", 8), 6: ("wedge", 6),
                7: ("pyramid", 5), 8: ("line3", 3), 9: ("triangle6", 6),
                11: ("tetra10", 10), 15: ("vertex", 1)}


def read_msh(filename):
    """Read a Gmsh ASCII MSH 2.x mesh (the format of PeriPy's ``.msh``
    examples, which it reads with meshio).

    Node coordinates come in file order; element node ids are mapped to
    those positions.  Elements are grouped by type in file order, as
    meshio's ``cells_dict`` groups them.

    :returns: :class:`Mesh`.
    :raises MeshFormatError: for binary or MSH 4 files and unknown element
        types.
    """
    lines = pathlib.Path(filename).read_text().splitlines()
    pos = 0

    def section(name):
        nonlocal pos
        while pos < len(lines) and lines[pos].strip() != name:
            pos += 1
        if pos == len(lines):
            raise MeshFormatError(f"{filename}: no {name} section")
        pos += 1

    section("$MeshFormat")
    version, file_type, _ = lines[pos].split()
    if not version.startswith("2"):
        raise MeshFormatError(f"{filename}: MSH {version} is not read "
                              "(MSH 2.x only)")
    if file_type != "0":
        raise MeshFormatError(f"{filename}: binary MSH is not read")
    section("$Nodes")
    nnodes = int(lines[pos])
    rows = np.array([ln.split() for ln in lines[pos + 1:pos + 1 + nnodes]],
                    dtype=np.float64).reshape(nnodes, 4)
    pos += 1 + nnodes
    ids = rows[:, 0].astype(np.int64)
    points = np.ascontiguousarray(rows[:, 1:4])
    index = np.full(int(ids.max()) + 1 if nnodes else 1, -1, dtype=np.int64)
    index[ids] = np.arange(nnodes)
    section("$Elements")
    nelem = int(lines[pos])
    groups = {}
    for ln in lines[pos + 1:pos + 1 + nelem]:
        v = ln.split()
        etype, ntags = int(v[1]), int(v[2])
        if etype not in MSH_ELEMENTS:
            raise MeshFormatError(f"{filename}: element type {etype}")
        name, nv = MSH_ELEMENTS[etype]
        nodes = [int(x) for x in v[3 + ntags:3 + ntags + nv]]
        groups.setdefault(name, []).append(nodes)
    cells_dict = {}
    for name, conn in groups.items():
        c = index[np.array(conn, dtype=np.int64)]
        if np.any(c < 0):
            raise MeshFormatError(f"{filename}: element refers to a "
                                  "missing node")
        cells_dict[name] = c
    return Mesh(points, cells_dict)


def read_mesh(filename):
    """Read a ``.msh`` (Gmsh MSH 2.x) or legacy ``.vtk`` mesh."""
    if str(filename).lower().endswith(".msh"):
        return read_msh(filename)
    return read_vtk(filename)
