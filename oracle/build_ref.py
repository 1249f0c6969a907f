"""Build recipe for ``oracle/_ref``: the reference heatsim2 package compiled from its own sources.

Test infrastructure only -- the product never imports anything under ``oracle/``.

The reference (isuthermography/heatsim2) is a Python package with three Cython extension modules
(heatsim2/tridiag.pyx, heatsim2/crank_nicolson.pyx, heatsim2/alternatingdirection_c_pyx.pyx, the last one
linked with the hand-written heatsim2/alternatingdirection_c.c).  Its shipped setup.py imports
numpy.distutils (setup.py:10), which numpy 2.x no longer has, so the reference's build system is not used.
This recipe instead:

  1. ``generate()`` (needs the reference sources and Cython; runs where the sources are mounted):
     cythonizes the three .pyx files (language_level=3) into ``oracle/_ref/gen/*.c`` and copies the
     package's pure-Python modules and the hand-written C/H files into ``oracle/_ref/heatsim2`` and
     ``oracle/_ref/gen``.  The reference's own Cython-0.29 generated .c files are not used.
  2. ``compile_generated()`` (needs only gcc, Python headers and numpy headers): compiles the generated
     C into ``oracle/_ref/heatsim2/*.so`` for the machine it runs on.

Everything is written under ``oracle/_ref`` (git-ignored).  Nothing under the reference tree is modified.
"""
import os
import shutil
import subprocess
import sys
import sysconfig
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
GEN = os.path.join(REF_OUT, "gen")
PKG = os.path.join(REF_OUT, "heatsim2")
DEFAULT_SRC = "/root/reference"

PYX_MODULES = {
    # module name -> (pyx file, extra hand-written C sources)
    "tridiag": ("tridiag.pyx", []),
    "crank_nicolson": ("crank_nicolson.pyx", []),
    "alternatingdirection_c_pyx": ("alternatingdirection_c_pyx.pyx", ["alternatingdirection_c.c"]),
}
PY_FILES = ["__init__.py", "expression.py", "boundary_insulating.py", "boundary_conducting.py",
            "boundary_conducting_anisotropic.py", "boundary_thininsulatinglayer.py",
            "tridiag_purepython.py", "surface_temperature.py"]
C_SUPPORT = ["alternatingdirection_c.c", "alternatingdirection_c.h", "cython_capsule_supp.h"]


def generate(src_root=DEFAULT_SRC):
    """Cythonize the reference's .pyx sources into oracle/_ref/gen (step 1)."""
    src_pkg = os.path.join(src_root, "heatsim2")
    if not os.path.isdir(src_pkg):
        raise FileNotFoundError(src_pkg)
    os.makedirs(GEN, exist_ok=True)
    os.makedirs(PKG, exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        tpkg = os.path.join(tmp, "heatsim2")
        os.makedirs(tpkg)
        for name in PY_FILES + C_SUPPORT + [v[0] for v in PYX_MODULES.values()]:
            shutil.copy(os.path.join(src_pkg, name), os.path.join(tpkg, name))
        for mod, (pyx, _extra) in PYX_MODULES.items():
            out_c = os.path.join(GEN, mod + ".c")
            subprocess.check_call([sys.executable, "-m", "cython", "-3", "--fast-fail",
                                   "-o", out_c, os.path.join(tpkg, pyx)], cwd=tmp)
        for name in C_SUPPORT:
            shutil.copy(os.path.join(tpkg, name), os.path.join(GEN, name))
        for name in PY_FILES:
            shutil.copy(os.path.join(tpkg, name), os.path.join(PKG, name))
    with open(os.path.join(PKG, "version.txt"), "w") as fh:
        fh.write("reference-built-from-pyx\n")


def compile_generated(jobs=3):
    """Compile oracle/_ref/gen/*.c into importable extension modules for this machine (step 2)."""
    import numpy
    if not os.path.isdir(GEN):
        raise FileNotFoundError(GEN)
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    inc = [sysconfig.get_paths()["include"], numpy.get_include(), GEN]
    procs = []
    for mod, (_pyx, extra) in PYX_MODULES.items():
        out = os.path.join(PKG, mod + ext)
        srcs = [os.path.join(GEN, mod + ".c")] + [os.path.join(GEN, e) for e in extra]
        cmd = ["gcc", "-shared", "-fPIC", "-O2", "-w", "-o", out] + srcs + \
              ["-I" + d for d in inc] + ["-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION"]
        procs.append(subprocess.Popen(cmd))
    rc = [p.wait() for p in procs]
    if any(rc):
        raise RuntimeError("compiling the reference extension modules failed: %r" % (rc,))


def available():
    """True when oracle/_ref holds an importable reference build for this machine."""
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    return all(os.path.exists(os.path.join(PKG, m + ext)) for m in PYX_MODULES)


def import_reference():
    """Import the reference package from oracle/_ref (adds oracle/_ref to sys.path)."""
    if REF_OUT not in sys.path:
        sys.path.insert(0, REF_OUT)
    import heatsim2  # noqa: F401  (the reference package)
    return sys.modules["heatsim2"]


def build(src_root=DEFAULT_SRC):
    """Generate (if the reference sources are present) and compile.  Returns True when usable."""
    if os.path.isdir(os.path.join(src_root, "heatsim2")):
        generate(src_root)
    if os.path.isdir(GEN):
        compile_generated()
    return available()


if __name__ == "__main__":
    ok = build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_SRC)
    print("oracle/_ref usable:", ok)
