"""The reference's PRIMME eigensolver, run from the oracle (test infrastructure).

``oracle/build_ref.py`` compiles tt-fort's vendored PRIMME C sources unchanged
into ``oracle/_ref/libprimme_ref.so`` together with ``primme_ref.c`` (BLAS
forwarders and a dprimme driver).  This module fills the forwarders from
scipy's cython_blas / cython_lapack tables and runs dprimme with the settings
of tt_eigb.f90:252-283:

  numEvals = B, method DYNAMIC (the reference's) or GD_plusK (deterministic:
  DYNAMIC switches between GD+k and JDQMR on wall-clock measurements,
  primme/main_iter_d.c:295-301,529-620), n, printLevel, maxMatvecs = 500,
  minRestartSize = min(B+1, n-1), maxBasisSize = 100, eps = eps2/resid_damp,
  initSize = B with the current block as the start.

``local_solver()`` returns a drop-in for the local eigensolver of
``oracle/eigb.py`` so that a whole tt_eigb sweep can run on PRIMME.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
METHODS = {"DYNAMIC": 0, "GD_plusK": 5, "JDQMR": 10}
_lib = None
_MV = C.CFUNCTYPE(None, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int)


def _capsule_ptr(cap):
    get_name = C.pythonapi.PyCapsule_GetName
    get_name.restype = C.c_char_p
    get_name.argtypes = [C.py_object]
    get_ptr = C.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = C.c_void_p
    get_ptr.argtypes = [C.py_object, C.c_char_p]
    return get_ptr(cap, get_name(cap))


def available():
    """True when libprimme_ref.so exists or can be built (the tt-fort source
    tree is present)."""
    try:
        lib()
        return True
    except (OSError, RuntimeError):
        return False


def lib():
    global _lib
    if _lib is not None:
        return _lib
    from . import build_ref
    path = build_ref.build()
    if path is None:
        raise RuntimeError("tt-fort source tree not found: libprimme_ref.so cannot be built")
    L = C.CDLL(path)
    L.ttref_set_fn.argtypes = [C.c_char_p, C.c_void_p]
    L.ttref_set_fn.restype = C.c_int
    L.ttref_blas_ready.restype = C.c_int
    L.ttref_dprimme.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int,
                                _MV, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]
    L.ttref_dprimme.restype = C.c_int
    import scipy.linalg.cython_blas as cb
    import scipy.linalg.cython_lapack as cl
    for name in ("dcopy", "dswap", "dgemm", "dsymm", "daxpy", "dgemv", "ddot", "dscal"):
        assert L.ttref_set_fn(name.encode(), _capsule_ptr(cb.__pyx_capi__[name])) == 0
    for name in ("dlarnv", "dsyev", "dsytrf", "dsytrs", "dlamch"):
        assert L.ttref_set_fn(name.encode(), _capsule_ptr(cl.__pyx_capi__[name])) == 0
    assert L.ttref_blas_ready() == 1
    _lib = L
    return _lib


def dprimme(mv, N, B, X0, eps, method="GD_plusK", max_matvecs=500, max_basis=100,
            print_level=0):
    """Lowest B eigenpairs of the operator mv (X (N x k) -> A X) by PRIMME,
    started from X0 (N x B).  Returns (evals, evecs, rnorms, matvecs, ierr)."""
    L = lib()
    evals = np.zeros(B)
    evecs = np.asfortranarray(np.array(X0, dtype=np.float64).reshape(N, B, order="F"))
    rnorms = np.zeros(B)
    err = []

    def cb(xp, yp, k):
        try:
            x = np.ctypeslib.as_array(xp, shape=(N * k,)).reshape(N, k, order="F")
            y = np.ctypeslib.as_array(yp, shape=(N * k,)).reshape(N, k, order="F")
            y[:, :] = mv(x.copy(order="F"))
        except Exception as e:   # an exception cannot cross the C frames
            err.append(e)

    cfun = _MV(cb)
    nmv = C.c_int(0)
    ierr = L.ttref_dprimme(N, B, METHODS[method], min(max_basis, N), max_matvecs, eps,
                           print_level, cfun, evals.ctypes.data, evecs.ctypes.data,
                           rnorms.ctypes.data, C.byref(nmv))
    if err:
        raise err[0]
    return evals, evecs, rnorms, nmv.value, ierr


def local_solver(method="GD_plusK", stats=None):
    """A local eigensolver for oracle/eigb.py's ``local_solver`` argument:
    (mv, X0, B, tol, max_matvecs) -> (lam, V, res, nmv).  PRIMME's ierr -3
    (maxMatvecs reached) is tolerated as tt_eigb.f90:285-288 does; any other
    negative ierr raises.  stats (a list) collects (N, nmv, ierr) per solve."""
    def solve(mv, X0, B, tol, max_matvecs):
        N = X0.shape[0]
        lam, V, rn, nmv, ierr = dprimme(mv, N, B, X0, tol, method=method,
                                        max_matvecs=max_matvecs)
        if ierr < 0 and ierr != -3:
            raise RuntimeError(f"dprimme failed with ierr={ierr}")
        if stats is not None:
            stats.append((N, nmv, ierr))
        return lam, V, float(np.linalg.norm(rn)), nmv
    return solve
