"""Compile the reference's own Cython CPU step into ``oracle/_ref`` (TEST
INFRASTRUCTURE: the checker and the timed CPU baseline, never the product).

Recipe
------
1. Where the reference checkout exists (read-only; the directory named by
   the ``PP_REFERENCE`` environment variable or the ``reference`` argument,
   else a ``reference`` directory beside this repository's checkout),
   Cython translates ``peripy/peridynamics.pyx``, ``peripy/correction.pyx``,
   ``peripy/create_crack.pyx`` and ``peripy/spatial.pyx`` (which the first
   two cimport through ``spatial.pxd``) from where they lie into C files under
   ``oracle/_ref/src/``.  Nothing is written
   into the reference tree and no reference source is copied.
2. gcc compiles each C file with the reference's own flags (``-O3``,
   ``setup.py:12``) plus ``-ffp-contract=off``, so that binary64 operations
   round one by one as written on every host (aarch64 gcc would otherwise
   fuse multiply-adds that the x86-64 build does not), into
   ``oracle/_ref/peripy/<module>.so``, importable as
   ``peripy.peridynamics`` / ``peripy.correction`` /
   ``peripy.create_crack`` / ``peripy.spatial`` once
   ``oracle/_ref`` is on
   ``sys.path`` (``oracle/_ref/peripy/__init__.py`` is an empty file written
   here so the package imports without the reference's own ``__init__``).

``oracle/_ref`` is git-ignored but travels to the GPU machine with the working
tree; there, without the reference checkout, step 1 is skipped and step 2
recompiles the generated C for the box's architecture.
"""
import os
import pathlib
import shutil
import subprocess
import sys
import sysconfig

HERE = pathlib.Path(__file__).resolve().parent
REF_OUT = HERE / "_ref"
SRC = REF_OUT / "src"
PKG = REF_OUT / "peripy"
MODULES = ("spatial", "peridynamics", "correction", "create_crack")
#: The reference checkout: ``$PP_REFERENCE``, else ``reference`` beside the
#: repository's own checkout.
DEFAULT_REFERENCE = pathlib.Path(
    os.environ.get("PP_REFERENCE") or HERE.parent.parent / "reference")


def _ext_suffix():
    return sysconfig.get_config_var("EXT_SUFFIX") or ".so"


def _cythonize(reference):
    """Generate C for each module from the reference sources."""
    from Cython.Compiler.Main import CompilationOptions, compile_single
    SRC.mkdir(parents=True, exist_ok=True)
    for name in MODULES:
        pyx = reference / "peripy" / f"{name}.pyx"
        out = SRC / f"{name}.c"
        opts = CompilationOptions(language_level=3, output_file=str(out))
        # The module's package (peripy) comes from the reference tree, so
        # `from .spatial cimport ...` resolves against peripy/spatial.pxd.
        compile_single(str(pyx), opts, full_module_name=f"peripy.{name}")


def _compile(quiet):
    PKG.mkdir(parents=True, exist_ok=True)
    (PKG / "__init__.py").write_text("")
    include = sysconfig.get_paths()["include"]
    cc = os.environ.get("CC", "gcc")
    for name in MODULES:
        src = SRC / f"{name}.c"
        out = PKG / f"{name}{_ext_suffix()}"
        if out.exists() and out.stat().st_mtime >= src.stat().st_mtime:
            continue
        cmd = [cc, "-O3", "-ffp-contract=off", "-shared", "-fPIC", "-I",
               include, str(src), "-o", str(out)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"compiling {src.name} failed:\n{res.stderr}")
        if not quiet:
            print("built", out)


def available():
    """True when the compiled reference modules exist for this Python."""
    return all((PKG / f"{n}{_ext_suffix()}").exists() for n in MODULES)


def build(reference=None, quiet=False):
    """Build ``oracle/_ref``; returns True when the modules are available.

    Without the reference checkout and without previously generated C the
    build is skipped (returns False): the compiled reference is optional
    test infrastructure.
    """
    reference = pathlib.Path(reference) if reference else DEFAULT_REFERENCE
    have_c = all((SRC / f"{n}.c").exists() for n in MODULES)
    if (reference / "peripy" / "peridynamics.pyx").exists():
        try:
            stale = not have_c or any(
                (reference / "peripy" / f"{n}.pyx").stat().st_mtime >
                (SRC / f"{n}.c").stat().st_mtime for n in MODULES)
            if stale:
                _cythonize(reference)
            have_c = True
        except ImportError:
            if not have_c:
                return False
    if not have_c or shutil.which(os.environ.get("CC", "gcc")) is None:
        return False
    if not pathlib.Path(sysconfig.get_paths()["include"], "Python.h").exists():
        return False
    _compile(quiet)
    return available()


def load(module="peridynamics"):
    """Import and return a compiled reference module (``peripy.<module>``)."""
    if not available():
        raise ImportError("oracle/_ref is not built")
    path = str(REF_OUT)
    if path not in sys.path:
        sys.path.insert(0, path)
    import importlib
    return importlib.import_module(f"peripy.{module}")


if __name__ == "__main__":
    ok = build(sys.argv[1] if len(sys.argv) > 1 else None)
    print("reference CPU step available:", ok)
