"""Build recipe for oracle/_ref/ (test infrastructure, not product).

Compiles the reference's vendored PRIMME eigensolver -- the real-valued C
sources of tt-fort's ``primme/`` directory, unchanged, read where they lie in
the tt-fort source tree -- together with this directory's ``primme_ref.c``
(BLAS forwarders + a dprimme driver with tt_eigb's settings) into
``oracle/_ref/libprimme_ref.so``.  Nothing is copied into the repository:
the sources are compiled in place and only the built objects land in
``oracle/_ref/`` (git-ignored).

  python oracle/build_ref.py [<tt-fort source tree>]

The source tree defaults to $TT_FORT_SRC, else /root/reference.  When it is
absent (for instance on a machine that only has this repository), build()
returns None and the PRIMME-pinned tests skip.

The reference's own build (Makefile + Makefile.in) generates int_redefine.h
from the integer preset; the i4 presets (Makefile.in:27-66) write
"// #define int long", i.e. C int stays 32-bit, which is what scipy's LP64
BLAS expects.  The same one-line header is generated here into
oracle/_ref/include.  zdotcsub.f (Fortran, complex only) and the complex
solver are not built: tt_eigb calls only dprimme.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libprimme_ref.so")

# real-valued PRIMME translation units (primme/Makefile.deps minus the
# complex ones, the Fortran-77 interface and zdotcsub.f)
PRIMME_D = ["common_numerical", "Complex", "convergence_d", "correction_d", "errors",
            "factorize_d", "init_d", "inner_solve_d", "locking_d", "main_iter_d", "numerical_d",
            "ortho_d", "primme_d", "primme_interface", "restart_d", "solve_H_d",
            "update_projection_d", "update_W_d", "wtime"]


def source_tree():
    root = os.environ.get("TT_FORT_SRC", "/root/reference")
    return root if os.path.isdir(os.path.join(root, "primme")) else None


def build(root=None, force=False):
    """Build oracle/_ref/libprimme_ref.so; returns its path, or None when the
    reference source tree is not present."""
    root = root or source_tree()
    if root is None:
        return None
    src = os.path.join(root, "primme")
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(os.path.join(src, f + ".c")) for f in PRIMME_D)
        newest = max(newest, os.path.getmtime(os.path.join(HERE, "primme_ref.c")))
        if os.path.getmtime(LIB) >= newest:
            return LIB
    cc = shutil.which("gcc") or "cc"
    inc = os.path.join(OUT, "include")
    obj = os.path.join(OUT, "obj")
    os.makedirs(inc, exist_ok=True)
    os.makedirs(obj, exist_ok=True)
    with open(os.path.join(inc, "int_redefine.h"), "w") as f:
        f.write("// #define int long\n")
    flags = ["-O2", "-fPIC", "-w", "-I", inc, "-I", src]

    def compile_one(path):
        o = os.path.join(obj, os.path.basename(path)[:-2] + ".o")
        r = subprocess.run([cc, "-c", path, "-o", o] + flags, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"gcc failed on {path}:\n{r.stderr}")
        return o

    paths = [os.path.join(src, f + ".c") for f in PRIMME_D] + [os.path.join(HERE, "primme_ref.c")]
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, paths))
    r = subprocess.run([cc, "-shared", "-o", LIB] + objs + ["-lm", "-Wl,--no-undefined"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


GMRES_LIB = os.path.join(OUT, "libgmres3d_ref.so")


def build_gmres3d(ttgpu_lib, root=None):
    """Compile tt-fort's gmres_3d.c (unchanged, from the source tree) with
    blas64_fwd.c and link it against the library's by-reference dbfun3 /
    djac_apply (ttgpu_lib) with every symbol resolved (--no-undefined).
    Returns the path of oracle/_ref/libgmres3d_ref.so, or None without the
    source tree."""
    root = root or source_tree()
    if root is None:
        return None
    cc = shutil.which("gcc") or "cc"
    obj = os.path.join(OUT, "obj")
    os.makedirs(obj, exist_ok=True)
    objs = []
    for path in (os.path.join(root, "gmres_3d.c"), os.path.join(HERE, "blas64_fwd.c")):
        o = os.path.join(obj, os.path.basename(path)[:-2] + ".o")
        r = subprocess.run([cc, "-c", path, "-o", o, "-O2", "-fPIC", "-w"], capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError(f"gcc failed on {path}:\n{r.stderr}")
        objs.append(o)
    libdir = os.path.dirname(os.path.abspath(ttgpu_lib))
    r = subprocess.run([cc, "-shared", "-o", GMRES_LIB] + objs +
                       ["-L" + libdir, "-l:" + os.path.basename(ttgpu_lib), "-Wl,-rpath," + libdir,
                        "-Wl,-Bsymbolic", "-lm", "-Wl,--no-undefined"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of gmres_3d.c against {ttgpu_lib} failed:\n{r.stderr}")
    return GMRES_LIB


if __name__ == "__main__":
    out = build(sys.argv[1] if len(sys.argv) > 1 else None, force=True)
    print(out or "tt-fort source tree not found; nothing built")
