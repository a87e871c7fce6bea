"""Recipe that compiles the reference C sources, in place, into oracle/_ref/.

Test infrastructure only.  The reference fixes its grid at compile time
(``input.h:45-47``), so one shared object is built per grid size from
``oracle/ref_harness.c`` + ``oracle/input.h`` with the reference headers taken
from the reference tree by ``-I``.  Outputs go only to ``oracle/_ref/``
(git-ignored).  Nothing is copied out of the reference tree.

FP flags: ``-O2 -ffp-contract=off`` so no multiply-add is fused (the GPU plain
FP64 build uses ``--fmad=false`` for the same reason); ``-mcmodel=medium``
because the reference's static arrays exceed 2 GB at 256x256x128.
``-Wl,-Bsymbolic`` binds the reference's globals to its own definitions: it
declares ``char dirname[64]`` (commontemp.h:183), which inside a shared object
would otherwise resolve to the C library's ``dirname()`` function.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REFERENCE_TREE = os.environ.get("MHD_REFERENCE_TREE", "/root/reference")


def available():
    return os.path.isfile(os.path.join(REFERENCE_TREE, "hlldx.h"))


def lib_path(nr, nphi, nz, shipped=False):
    return os.path.join(OUT, "libref_%s%dx%dx%d.so" % ("shipped_" if shipped else "", nr, nphi, nz))


def build(nr, nphi, nz, force=False, shipped=False):
    """Build (if needed) and return the path of the reference library for one
    grid: the uniform disc grid, or (shipped) the reference's stretched grid."""
    if not available():
        raise FileNotFoundError("reference tree not present: %s" % REFERENCE_TREE)
    os.makedirs(OUT, exist_ok=True)
    out = lib_path(nr, nphi, nz, shipped)
    src = os.path.join(HERE, "ref_harness.c")
    inp = os.path.join(HERE, "input.h")
    if (not force and os.path.exists(out)
            and os.path.getmtime(out) >= max(os.path.getmtime(src), os.path.getmtime(inp),
                                              os.path.getmtime(os.path.abspath(__file__)))):
        return out
    cmd = ["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-fPIC", "-shared", "-mcmodel=medium", "-Wl,-Bsymbolic",
           "-w", "-Wno-implicit-function-declaration",
           "-DREF_NR=%d" % nr, "-DREF_NPHI=%d" % nphi, "-DREF_NZ=%d" % nz]
    if shipped:
        cmd.append("-DREF_SHIPPED")
    cmd += ["-I", HERE, "-I", REFERENCE_TREE, src, "-o", out + ".tmp", "-lm"]
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    sizes = [tuple(int(v) for v in a.split("x")) for a in sys.argv[1:]] or [(64, 64, 32)]
    for s in sizes:
        print(build(*s))
