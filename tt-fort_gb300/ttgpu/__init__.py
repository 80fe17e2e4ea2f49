"""Python mirror of the tt-fort sweep interface, backed by libttgpu.so (CUDA).

Driver calls mirror the reference's Fortran entry points and argument meaning:

  tt_eigb(d, n, m, ra, crA, crY0, ry, eps, rmax, B, ...)      tt_eigb.f90:110
  ztt_ksl(d, n, m, ra, crA, crY0, ry, tau, rmax, ...)        tt_ksl.f90:431
  tt_amen_solve(d, n, m, ry, ra, crA, crY, crX0, rx, eps, ...) tt_adapt_als.f90:513

They take host (numpy) arrays in the reference's flat column-major layout and
return the result cores (the reference's module array ``result_core``) with
the updated ranks.  Kernel-level calls (``dbfun3``, ``dphi_left`` ...) take
torch CUDA tensors and run on the device.  There is no CPU fallback: every
call goes through the CUDA library, and importing fails loudly when the
library has not been built.
"""
import ctypes as C
import os

import numpy as np

from . import operators  # noqa: F401  (input builders)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libttgpu.so")

TTG_OK = 0
TTG_ERR_ARG = -1
TTG_ERR_NOCONV = -4
TTG_ERR_UNSUPPORTED = -7
METHOD = {"plain": 0, "split": 1, "jd64": 2}

_i64 = C.c_int64
_i64p = C.POINTER(C.c_int64)
_dp = C.c_void_p
_lib = None


class TTGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"ttgpu error {code}: {msg}")
        self.code = code


def lib():
    """Load libttgpu.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with tt-fort_gb300/ttgpu/build.py "
                "(or __graft_entry__.build()); there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        L.ttg_last_error.restype = C.c_char_p
        L.ttg_last_error.argtypes = [C.c_void_p]
        L.ttg_my_chop3.restype = _i64
        L.ttg_my_chop3.argtypes = [_i64, C.c_void_p, C.c_double]
        L.ttg_launch_count.restype = _i64
        L.ttg_djac_size.restype = _i64
        L.ttg_djac_size.argtypes = [C.c_char, _i64, _i64, _i64]
        L.ttg_mlp_nparams.restype = _i64
        L.ttg_mlp_nparams.argtypes = [C.c_void_p]
        L.ttg_capped.restype = _i64
        L.ttg_capped.argtypes = [C.c_void_p]
        _lib = L
    return _lib


# every symbol declared in include/ttgpu.h
EXPORTED = [
    "ttg_create", "ttg_destroy", "ttg_last_error", "ttg_set_stream", "ttg_synchronize",
    "ttg_version", "ttg_dbfun3", "ttg_dbfun3_split", "ttg_dbfun3_noalloc", "ttg_zbfun3", "ttg_zbfun3_transp",
    "ttg_dphi_left", "ttg_dphi_right", "ttg_zphi_left", "ttg_zphi_right", "ttg_dphi2_left",
    "ttg_dphi2_right", "ttg_d2d_fullmat", "ttg_dqr", "ttg_zqr", "ttg_dsyev", "ttg_dgesvd",
    "ttg_my_chop3", "ttg_dmaxvol", "ttg_eigb", "ttg_ksl_z", "ttg_amen_solve", "ttg_dtt_amen_solve",
    "ttg_result_size", "ttg_result_copy", "ttg_zresult_copy", "ttg_free_result", "ttg_stats",
    "ttg_launch_count", "ttg_localop_create", "ttg_localop_apply", "ttg_localop_destroy",
    "ttg_mlp_create", "ttg_mlp_destroy", "ttg_mlp_nparams", "ttg_mlp_get_params",
    "ttg_mlp_set_params", "ttg_mlp_get_grads", "ttg_mlp_forward", "ttg_mlp_loss_grad",
    "ttg_mlp_adam_step", "ttg_set_learned", "ttg_record_count", "ttg_record_clear",
    "ttg_mlp_train_recorded", "ttg_batch_create", "ttg_batch_destroy", "ttg_batch_add_eigb",
    "ttg_batch_run", "ttg_batch_result", "ttg_batch_cores", "ttg_djac_size", "ttg_djac_gen",
    "ttg_djac_apply", "ttg_mvk4", "ttg_sdv_write", "ttg_sdv_read", "ttg_diag_ksl_z",
    "ttg_diag_ksl_d", "ttg_ksl_d", "ttg_set_limits", "ttg_capped",
    "ttg_local_eig", "dbfun3", "djac_gen", "djac_apply", "dqr", "ttg_fshim_status",
    "ttg_mlp_set_precision", "ttg_mlp_check",
]


class Context:
    """Owns a ttg_ctx (one per host thread), i.e. the reference's module state."""

    def __init__(self, device=0):
        self._h = C.c_void_p()
        rc = lib().ttg_create(C.c_int(device), C.byref(self._h))
        if rc != TTG_OK:
            raise TTGError(rc, "ttg_create failed (is a CUDA device visible?)")

    @property
    def handle(self):
        return self._h

    def check(self, rc):
        if rc != TTG_OK:
            raise TTGError(rc, lib().ttg_last_error(self._h).decode())

    def synchronize(self):
        self.check(lib().ttg_synchronize(self._h))

    def set_stream(self, stream_ptr):
        self.check(lib().ttg_set_stream(self._h, C.c_void_p(stream_ptr)))
        self._stream = stream_ptr

    def bind_torch_stream(self):
        """Run subsequent calls on torch's current CUDA stream, so that the
        caching allocator's stream-ordered reuse of tensor memory is safe."""
        import torch
        s = torch.cuda.current_stream().cuda_stream
        if getattr(self, "_stream", None) != s:
            self.set_stream(s)

    def stats(self):
        mv, sw, la = _i64(), _i64(), _i64()
        res = C.c_double()
        lib().ttg_stats(self._h, C.byref(mv), C.byref(sw), C.byref(res), C.byref(la))
        return {"matvecs": mv.value, "sweeps": sw.value, "res": res.value, "launches": la.value}

    def set_limits(self, max_matvecs=0, max_expokit_steps=0, strict=False):
        """Iteration caps of the local solvers for the next driver calls (0 =
        the reference's 500 / 500).  strict=True turns a capped local solve
        into TTGError(TTG_ERR_NOCONV); otherwise it is tolerated and counted,
        as the reference tolerates PRIMME's -3 and Expokit's iflag = 1."""
        if max_matvecs < 0 or max_expokit_steps < 0:
            raise ValueError("caps must be >= 0")
        self.check(lib().ttg_set_limits(self._h, _i64(max_matvecs), _i64(max_expokit_steps),
                                        C.c_int(1 if strict else 0)))

    def capped(self):
        """Local solves of the last driver call that stopped at a cap."""
        return int(lib().ttg_capped(self._h))

    def close(self):
        if self._h:
            lib().ttg_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def launch_count():
    return int(lib().ttg_launch_count())


def _iarr(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.int64))


def _darr(v):
    """float64 copy of a real array; complex input is an error (a real entry
    point would otherwise drop the imaginary parts)."""
    a = np.asarray(v)
    if np.iscomplexobj(a):
        raise TypeError("this entry point takes real arrays; use the complex one (z...) instead")
    return np.ascontiguousarray(a, dtype=np.float64)


def _carr(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.complex128))


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _dev(t, need=0, dtype=None, what="tensor"):
    """Device pointer of a torch CUDA tensor (contiguous).  With ``dtype``
    ("float64", "complex128", "int64") the element type is checked, and
    ``need`` is the least number of elements the call reads or writes: the
    kernels take bare pointers, so a short tensor is an argument error
    (TTG_ERR_ARG) here rather than an out-of-bounds access on the device."""
    if not getattr(t, "is_cuda", False):
        raise TypeError("kernel-level calls take torch CUDA tensors")
    if not t.is_contiguous():
        raise ValueError("tensor must be contiguous")
    if dtype is not None and str(t.dtype) != "torch." + dtype:
        raise TypeError(f"{what}: {t.dtype}, torch.{dtype} expected")
    if t.numel() < int(need):
        raise TTGError(TTG_ERR_ARG, f"{what}: {t.numel()} elements, the sizes need {int(need)}")
    return C.c_void_p(t.data_ptr())


def _bfun3_ptrs(dims, phi1, A, phi2, x, y, nvec, dtype, transp=False):
    """Checked pointers of a local product y = Phi1 A Phi2 x: phi1 (ry1, rx1,
    ra1), A (ra1, n, m, ra2), phi2 (rx2, ra2, ry2), x (rx1, m, rx2) and y
    (ry1, n, ry2) per vector; the adjoint swaps the shapes of x and y."""
    rx1, m, rx2, ry1, n, ry2, ra1, ra2 = (int(v) for v in dims)
    nx, ny = rx1 * m * rx2 * int(nvec), ry1 * n * ry2 * int(nvec)
    if transp:
        nx, ny = ny, nx
    return (_dev(phi1, ry1 * rx1 * ra1, dtype, "phi1"), _dev(A, ra1 * n * m * ra2, dtype, "A"),
            _dev(phi2, rx2 * ra2 * ry2, dtype, "phi2"), _dev(x, nx, dtype, "x"),
            _dev(y, ny, dtype, "y"))


def _tt_len(d, r, n, m=None):
    """Entries of packed TT cores r[k] x n[k] (x m[k]) x r[k+1], k < d."""
    return sum(int(r[k]) * int(n[k]) * (int(m[k]) if m is not None else 1) * int(r[k + 1])
               for k in range(d))


def _check_sizes(name, d, modes, ranks, arrays):
    """Host-side checks before a driver call: the C entry points take bare
    pointers (as the reference's assumed-size arrays), so a short array
    would be read past its end.  modes/ranks: {label: array} that need d
    resp. d + 1 entries; arrays: (label, array, r, n[, m]), the array holding
    packed cores r[k] x n[k] (x m[k]) x r[k+1].  Failures
    raise TTGError with TTG_ERR_ARG, the code the library returns for its own
    argument checks."""
    d = int(d)
    if d < 1:
        raise TTGError(TTG_ERR_ARG, f"{name}: d must be >= 1")
    for label, a in modes.items():
        if len(a) < d:
            raise TTGError(TTG_ERR_ARG, f"{name}: {label} has {len(a)} entries, d = {d} needed")
    for label, a in ranks.items():
        if len(a) < d + 1:
            raise TTGError(TTG_ERR_ARG,
                           f"{name}: {label} has {len(a)} entries, d + 1 = {d + 1} needed")
    for label, a, *dims in arrays:
        need = _tt_len(d, *dims)
        if a.size < need:
            raise TTGError(TTG_ERR_ARG,
                           f"{name}: {label} has {a.size} entries, the sizes need {need}")


# ------------------------------------------------------------------ drivers
def tt_eigb(d, n, m, ra, crA, crY0, ry, eps, rmax, B, kickrank=None, nswp=20,
            max_full_size=2000, verb=0, method="plain", ctx=None):
    """Block eigensolver (tt_eigb.f90:110).  Returns (lambda, cores, ry).

    ``kickrank`` is accepted and ignored, as in the reference (unused there).
    """
    n_, m_, ra_ = _iarr(n), _iarr(m), _iarr(ra)
    ry_ = _iarr(ry).copy()
    A_, Y_ = _darr(crA), _darr(crY0)
    _check_sizes("tt_eigb", d, {"n": n_, "m": m_}, {"ra": ra_, "ry": ry_},
                 [("crA", A_, ra_, n_, m_), ("crY0", Y_, ry_, n_)])
    ctx = ctx or default_context()
    lam = np.zeros(int(B))
    rc = lib().ttg_eigb(ctx.handle, _i64(d), _p(n_), _p(m_), _p(ra_), _p(A_), _p(Y_), _p(ry_),
                        C.c_double(eps), _i64(rmax), _p(lam), _i64(B), _i64(nswp),
                        _i64(max_full_size), C.c_int(verb), C.c_int(METHOD[method]))
    ctx.check(rc)
    return lam, _result(ctx, real=True), [int(v) for v in ry_]


def ztt_ksl(d, n, m, ra, crA, crY0, ry, tau, rmax, kickrank=None, nswp=None, verb=0, typ=2,
            order=8, method="plain", nsteps=1, ctx=None):
    """KSL time stepping (ztt_ksl, tt_ksl.f90:431): ``nsteps`` consecutive
    steps of size tau on the device.  Returns (cores, ry)."""
    n_, m_, ra_ = _iarr(n), _iarr(m), _iarr(ra)
    ry_ = _iarr(ry).copy()
    A_, Y_ = _carr(crA), _carr(crY0)
    _check_sizes("ztt_ksl", d, {"n": n_, "m": m_}, {"ra": ra_, "ry": ry_},
                 [("crA", A_, ra_, n_, m_), ("crY0", Y_, ry_, n_)])
    ctx = ctx or default_context()
    rc = lib().ttg_ksl_z(ctx.handle, _i64(d), _p(n_), _p(m_), _p(ra_), _p(A_), _p(Y_), _p(ry_),
                         C.c_double(tau), _i64(rmax), C.c_int(verb), C.c_int(typ),
                         C.c_int(order), C.c_int(METHOD[method]), _i64(nsteps))
    ctx.check(rc)
    return _result(ctx, real=False), [int(v) for v in ry_]


def tt_ksl(d, n, m, ra, crA, crY0, ry, tau, rmax, kickrank=None, nswp=None, verb=0, typ=2,
           order=8, method="plain", nsteps=1, ctx=None):
    """KSL time stepping with real data (tt_ksl, tt_ksl.f90:191): the real
    routine's sweep, ``nsteps`` consecutive steps on the device.  Returns
    (cores, ry), real."""
    n_, m_, ra_ = _iarr(n), _iarr(m), _iarr(ra)
    ry_ = _iarr(ry).copy()
    A_, Y_ = _darr(crA), _darr(crY0)
    _check_sizes("tt_ksl", d, {"n": n_, "m": m_}, {"ra": ra_, "ry": ry_},
                 [("crA", A_, ra_, n_, m_), ("crY0", Y_, ry_, n_)])
    ctx = ctx or default_context()
    rc = lib().ttg_ksl_d(ctx.handle, _i64(d), _p(n_), _p(m_), _p(ra_), _p(A_), _p(Y_), _p(ry_),
                         C.c_double(tau), _i64(rmax), C.c_int(verb), C.c_int(typ),
                         C.c_int(order), C.c_int(METHOD[method]), _i64(nsteps))
    ctx.check(rc)
    return _result(ctx, real=True), [int(v) for v in ry_]


def sdv_write(path, n, r, cores, complex_=False):
    """Write a TT tensor in the reference's .sdv format (dtt_write / ztt_write,
    ttio.f90:29-192); cores flat, column-major, float64 or complex128."""
    n_, r_ = _iarr(n), _iarr(r)
    c = np.ascontiguousarray(cores, dtype=np.complex128 if complex_ else np.float64)
    if len(r_) != len(n_) + 1:
        raise ValueError("sdv_write: r needs len(n) + 1 entries")
    if len(n_) < 1 or (n_ < 1).any() or (r_ < 1).any():
        raise ValueError("sdv_write: mode sizes and ranks must be positive")
    need = sum(int(r_[k]) * int(n_[k]) * int(r_[k + 1]) for k in range(len(n_)))
    if c.size != need:
        raise ValueError(f"sdv_write: {c.size} core entries, the ranks need {need}")
    rc = lib().ttg_sdv_write(str(path).encode(), _i64(len(n_)), _p(n_), _p(r_),
                             c.ctypes.data_as(C.c_void_p), C.c_int(1 if complex_ else 0))
    if rc != 0:
        raise RuntimeError(f"ttg_sdv_write failed ({rc}): {path}")


def sdv_read(path, complex_=False):
    """Read a .sdv file (dtt_read / ztt_read, ttio.f90:196-399): (n, r, cores)."""
    d = C.c_int64(0)
    ne = C.c_int64(0)
    rc = lib().ttg_sdv_read(str(path).encode(), C.c_int(int(complex_)), C.byref(d), None, None,
                            _i64(0), None, C.byref(ne))
    if rc != 0:
        raise RuntimeError(f"ttg_sdv_read failed ({rc}): {path}")
    n_ = np.zeros(d.value, dtype=np.int64)
    r_ = np.zeros(d.value + 1, dtype=np.int64)
    cores = np.zeros(ne.value, dtype=np.complex128 if complex_ else np.float64)
    rc = lib().ttg_sdv_read(str(path).encode(), C.c_int(int(complex_)), C.byref(d), _p(n_), _p(r_),
                            _i64(d.value), cores.ctypes.data_as(C.c_void_p), C.byref(ne))
    if rc != 0:
        raise RuntimeError(f"ttg_sdv_read failed ({rc}): {path}")
    return [int(v) for v in n_], [int(v) for v in r_], cores


def tt_mvk4(d, n, m, rx, ra, crA, crX, crY0, ry, eps, rmax, kickrank=5, nswp=20, verb=0,
            ctx=None):
    """AMEn matvec y ~ A x (tt_mvk4, tt_adapt_als.f90:67).  Returns (cores, ry)."""
    n_, m_, rx_, ra_ = _iarr(n), _iarr(m), _iarr(rx), _iarr(ra)
    ry_ = _iarr(ry).copy()
    A_, X_, Y_ = _darr(crA), _darr(crX), _darr(crY0)
    _check_sizes("tt_mvk4", d, {"n": n_, "m": m_}, {"rx": rx_, "ra": ra_, "ry": ry_},
                 [("crA", A_, ra_, n_, m_), ("crX", X_, rx_, m_),
                  ("crY0", Y_, ry_, n_)])
    ctx = ctx or default_context()
    rc = lib().ttg_mvk4(ctx.handle, _i64(d), _p(n_), _p(m_), _p(rx_), _p(ra_), _p(A_), _p(X_),
                        _p(Y_), _p(ry_), C.c_double(eps), _i64(rmax), _i64(kickrank), _i64(nswp),
                        C.c_int(verb))
    ctx.check(rc)
    return _result(ctx, real=True), [int(v) for v in ry_]


def tt_diag_ksl(d, n, ra, crA, crY0, ry, tau, rmax, verb=0, typ=2, order=8, nsteps=1,
                ctx=None):
    """KSL for an operator diagonal in the physical index (ztt_diag_ksl /
    dtt_diag_ksl, tt_diag_ksl.f90:315,560): crA holds cores A(a1, i, a2).
    Complex inputs run ztt_diag_ksl, real ones dtt_diag_ksl.  Returns (cores, ry)."""
    cplx = np.iscomplexobj(crA) or np.iscomplexobj(crY0)
    n_, ra_ = _iarr(n), _iarr(ra)
    ry_ = _iarr(ry).copy()
    A_, Y_ = (_carr(crA), _carr(crY0)) if cplx else (_darr(crA), _darr(crY0))
    _check_sizes("tt_diag_ksl", d, {"n": n_}, {"ra": ra_, "ry": ry_},
                 [("crA", A_, ra_, n_), ("crY0", Y_, ry_, n_)])
    ctx = ctx or default_context()
    f = lib().ttg_diag_ksl_z if cplx else lib().ttg_diag_ksl_d
    rc = f(ctx.handle, _i64(d), _p(n_), _p(ra_), _p(A_), _p(Y_), _p(ry_), C.c_double(tau),
           _i64(rmax), C.c_int(verb), C.c_int(typ), C.c_int(order), _i64(nsteps))
    ctx.check(rc)
    return _result(ctx, real=not cplx), [int(v) for v in ry_]


def tt_amen_solve(d, n, m, ry, ra, crA, crY, crX0, rx, eps, kickrank=4, nswp=20, verb=0,
                  prec="n", nrestart=40, niters=2, rmax=0, method="plain", ctx=None):
    """AMEn solve A x = y (tt_amen_solve, tt_adapt_als.f90:513).  Returns (cores, rx)."""
    n_, m_, ry_, ra_ = _iarr(n), _iarr(m), _iarr(ry), _iarr(ra)
    rx_ = _iarr(rx).copy()
    A_, Y_, X_ = _darr(crA), _darr(crY), _darr(crX0)
    _check_sizes("tt_amen_solve", d, {"n": n_, "m": m_}, {"ry": ry_, "ra": ra_, "rx": rx_},
                 [("crA", A_, ra_, n_, m_), ("crY", Y_, ry_, n_),
                  ("crX0", X_, rx_, m_)])
    ctx = ctx or default_context()
    rc = lib().ttg_amen_solve(ctx.handle, _i64(d), _p(n_), _p(m_), _p(ry_), _p(ra_), _p(A_),
                              _p(Y_), _p(X_), _p(rx_), C.c_double(eps), _i64(kickrank),
                              _i64(nswp), C.c_int(verb), C.c_char(prec.encode()),
                              _i64(nrestart), _i64(niters), _i64(rmax), C.c_int(METHOD[method]))
    ctx.check(rc)
    return _result(ctx, real=True), [int(v) for v in rx_]


def dtt_amen_solve(d, n, m, ry, ra, crA, crY, crX0, rx, eps, rmax=1000, kickrank=4, nswp=20,
                   verb=0, method="plain", ctx=None):
    """AMEn solve of ttamen.f90 (dtt_amen_solve, ttamen.f90:29) on packed cores.
    Returns (cores, rx)."""
    n_, m_, ry_, ra_ = _iarr(n), _iarr(m), _iarr(ry), _iarr(ra)
    rx_ = _iarr(rx).copy()
    A_, Y_, X_ = _darr(crA), _darr(crY), _darr(crX0)
    _check_sizes("dtt_amen_solve", d, {"n": n_, "m": m_}, {"ry": ry_, "ra": ra_, "rx": rx_},
                 [("crA", A_, ra_, n_, m_), ("crY", Y_, ry_, n_),
                  ("crX0", X_, rx_, m_)])
    ctx = ctx or default_context()
    rc = lib().ttg_dtt_amen_solve(ctx.handle, _i64(d), _p(n_), _p(m_), _p(ry_), _p(ra_), _p(A_),
                                  _p(Y_), _p(X_), _p(rx_), C.c_double(eps), _i64(rmax),
                                  _i64(kickrank), _i64(nswp), C.c_int(verb),
                                  C.c_int(METHOD[method]))
    ctx.check(rc)
    return _result(ctx, real=True), [int(v) for v in rx_]


def _result(ctx, real=True):
    nel = _i64()
    lib().ttg_result_size(ctx.handle, C.byref(nel))
    if real:
        out = np.zeros(nel.value)
        ctx.check(lib().ttg_result_copy(ctx.handle, _p(out), nel))
    else:
        out = np.zeros(nel.value, dtype=np.complex128)
        ctx.check(lib().ttg_zresult_copy(ctx.handle, _p(out), nel))
    lib().ttg_free_result(ctx.handle)
    return out


def my_chop3(s, eps):
    s_ = _darr(s)
    return int(lib().ttg_my_chop3(_i64(len(s_)), _p(s_), C.c_double(eps)))


# ------------------------------------------------------- kernel level (torch)
def _dims(*v):
    return [_i64(int(x)) for x in v]


def _kctx(ctx):
    ctx = ctx or default_context()
    ctx.bind_torch_stream()
    return ctx


def dbfun3(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, x, y, nvec=1, split=False,
           ctx=None):
    """y = Phi1 A Phi2 x on the device (dbfun3, ttals.f90:9); torch CUDA tensors."""
    dims = (rx1, m, rx2, ry1, n, ry2, ra1, ra2)
    ptrs = _bfun3_ptrs(dims, phi1, A, phi2, x, y, nvec, "float64")
    ctx = _kctx(ctx)
    f = lib().ttg_dbfun3_split if split else lib().ttg_dbfun3
    ctx.check(f(ctx.handle, *_dims(*dims), *ptrs, _i64(nvec)))


def local_eig(r1, n, r2, ra1, ra2, phi1, A, phi2, X, B, tol, max_matvecs=500, method="plain",
              ctx=None):
    """Lowest B eigenpairs of the local operator y = Phi1 A Phi2 x (the
    dprimme call of tt_eigb, tt_eigb.f90:252-283) on device tensors: X
    (N x B) holds the start block and receives the Ritz vectors.  Returns
    (lambda, res, matvecs)."""
    N = int(r1) * int(n) * int(r2)
    dims = (r1, n, r2, r1, n, r2, ra1, ra2)
    ptrs = _bfun3_ptrs(dims, phi1, A, phi2, X, X, B, "float64")
    ctx = _kctx(ctx)
    lam = np.zeros(int(B))
    res = C.c_double()
    nmv = _i64()
    ctx.check(lib().ttg_local_eig(ctx.handle, *_dims(r1, n, r2, ra1, ra2), ptrs[0], ptrs[1],
                                  ptrs[2], ptrs[3], _i64(B), C.c_double(tol), _i64(max_matvecs),
                                  C.c_int(METHOD[method]), _p(lam), C.byref(res),
                                  C.byref(nmv)))
    assert N >= B
    return lam, res.value, nmv.value


def djac_size(ptype, rx1, n, rx2):
    """Doubles of the block-Jacobi preconditioner (djac_gen, tt_linalg.f90:363)."""
    return int(lib().ttg_djac_size(ptype.encode(), rx1, n, rx2))


def djac_gen(ptype, rx1, n, rx2, ra1, ra2, phi1, A, phi2, jacs, ctx=None):
    """Block-Jacobi blocks of the local system into jacs (djac_gen,
    tt_linalg.f90:363-494); torch CUDA tensors."""
    ptrs = (_dev(phi1, rx1 * rx1 * ra1, "float64", "phi1"),
            _dev(A, ra1 * n * n * ra2, "float64", "A"),
            _dev(phi2, rx2 * ra2 * rx2, "float64", "phi2"),
            _dev(jacs, max(0, djac_size(ptype, rx1, n, rx2)), "float64", "jacs"))
    ctx = _kctx(ctx)
    ctx.check(lib().ttg_djac_gen(ctx.handle, C.c_char(ptype.encode()), _i64(rx1), _i64(n),
                                 _i64(rx2), _i64(ra1), _i64(ra2), *ptrs))


def djac_apply(ptype, rx1, n, rx2, jacs, x, y, ctx=None):
    """y = P x with the blocks of djac_gen (djac_apply, tt_linalg.f90:497-531)."""
    nx = rx1 * n * rx2
    ptrs = (_dev(jacs, max(0, djac_size(ptype, rx1, n, rx2)), "float64", "jacs"),
            _dev(x, nx, "float64", "x"), _dev(y, nx, "float64", "y"))
    ctx = _kctx(ctx)
    ctx.check(lib().ttg_djac_apply(ctx.handle, C.c_char(ptype.encode()), _i64(rx1), _i64(n),
                                   _i64(rx2), *ptrs))


def zbfun3(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, x, y, nvec=1, transp=False,
           ctx=None):
    """Complex product zbfun3 (ttals.f90:34) / zbfun3_transp (:85); complex128 tensors."""
    dims = (rx1, m, rx2, ry1, n, ry2, ra1, ra2)
    ptrs = _bfun3_ptrs(dims, phi1, A, phi2, x, y, nvec, "complex128", transp=transp)
    ctx = _kctx(ctx)
    f = lib().ttg_zbfun3_transp if transp else lib().ttg_zbfun3
    ctx.check(f(ctx.handle, *_dims(*dims), *ptrs, _i64(nvec)))


def phi_left(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1_old, A, x, y, out, complex_=False,
             ctx=None):
    dt = "complex128" if complex_ else "float64"
    ptrs = (_dev(phi1_old, ry1 * rx1 * ra1, dt, "phi1_old"), _dev(A, ra1 * n * m * ra2, dt, "A"),
            _dev(x, rx1 * m * rx2, dt, "x"), _dev(y, ry1 * n * ry2, dt, "y"),
            _dev(out, ry2 * rx2 * ra2, dt, "out"))
    ctx = _kctx(ctx)
    f = lib().ttg_zphi_left if complex_ else lib().ttg_dphi_left
    ctx.check(f(ctx.handle, *_dims(rx1, m, rx2, ry1, n, ry2, ra1, ra2), *ptrs))


def phi_right(rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi2_old, A, x, y, out, complex_=False,
              ctx=None):
    dt = "complex128" if complex_ else "float64"
    ptrs = (_dev(phi2_old, rx2 * ra2 * ry2, dt, "phi2_old"), _dev(A, ra1 * n * m * ra2, dt, "A"),
            _dev(x, rx1 * m * rx2, dt, "x"), _dev(y, ry1 * n * ry2, dt, "y"),
            _dev(out, rx1 * ra1 * ry1, dt, "out"))
    ctx = _kctx(ctx)
    f = lib().ttg_zphi_right if complex_ else lib().ttg_dphi_right
    ctx.check(f(ctx.handle, *_dims(rx1, m, rx2, ry1, n, ry2, ra1, ra2), *ptrs))


def phi2_left(rx1, rx2, ry1, n, ry2, phi1_old, x, y, out, ctx=None):
    ptrs = (_dev(phi1_old, ry1 * rx1, "float64", "phi1_old"),
            _dev(x, rx1 * n * rx2, "float64", "x"), _dev(y, ry1 * n * ry2, "float64", "y"),
            _dev(out, ry2 * rx2, "float64", "out"))
    ctx = _kctx(ctx)
    ctx.check(lib().ttg_dphi2_left(ctx.handle, *_dims(rx1, rx2, ry1, n, ry2), *ptrs))


def phi2_right(rx1, rx2, ry1, n, ry2, phi2_old, x, y, out, ctx=None):
    ptrs = (_dev(phi2_old, rx2 * ry2, "float64", "phi2_old"),
            _dev(x, rx1 * n * rx2, "float64", "x"), _dev(y, ry1 * n * ry2, "float64", "y"),
            _dev(out, rx1 * ry1, "float64", "out"))
    ctx = _kctx(ctx)
    ctx.check(lib().ttg_dphi2_right(ctx.handle, *_dims(rx1, rx2, ry1, n, ry2), *ptrs))


def fullmat(rx1, m, rx2, ra1, ra2, phi1, A, phi2, out, ctx=None):
    N = rx1 * m * rx2
    ptrs = (_dev(phi1, rx1 * rx1 * ra1, "float64", "phi1"),
            _dev(A, ra1 * m * m * ra2, "float64", "A"),
            _dev(phi2, rx2 * ra2 * rx2, "float64", "phi2"), _dev(out, N * N, "float64", "out"))
    ctx = _kctx(ctx)
    ctx.check(lib().ttg_d2d_fullmat(ctx.handle, *_dims(rx1, m, rx2, ra1, ra2), *ptrs))


def dqr(nrows, ncols, A, R, complex_=False, ctx=None):
    """In-place QR (dqr matrix_util.f90:37): A -> Q, R written."""
    dt = "complex128" if complex_ else "float64"
    ptrs = (_dev(A, nrows * ncols, dt, "A"), _dev(R, min(nrows, ncols) * ncols, dt, "R"))
    ctx = _kctx(ctx)
    f = lib().ttg_zqr if complex_ else lib().ttg_dqr
    ctx.check(f(ctx.handle, _i64(nrows), _i64(ncols), *ptrs))


def dsyev(k, A, w, ctx=None):
    ptrs = (_dev(A, k * k, "float64", "A"), _dev(w, k, "float64", "w"))
    ctx = _kctx(ctx)
    ctx.check(lib().ttg_dsyev(ctx.handle, _i64(k), *ptrs))


def dgesvd(p, q, M, U, s, Vt, ctx=None):
    r = min(p, q)
    ptrs = (_dev(M, p * q, "float64", "M"), _dev(U, p * r, "float64", "U"),
            _dev(s, r, "float64", "s"), _dev(Vt, r * q, "float64", "Vt"))
    ctx = _kctx(ctx)
    ctx.check(lib().ttg_dgesvd(ctx.handle, _i64(p), _i64(q), *ptrs))


def dmaxvol(nrows, r, A, p, Z=None, tol=1e-2, maxiters=1024, ctx=None):
    ptrs = (_dev(A, nrows * r, "float64", "A"), _dev(p, r, "int64", "p"),
            _dev(Z, nrows * r, "float64", "Z") if Z is not None else C.c_void_p())
    ctx = _kctx(ctx)
    ctx.check(lib().ttg_dmaxvol(ctx.handle, _i64(nrows), _i64(r), *ptrs, C.c_double(tol),
                                _i64(maxiters)))


class LocalOp:
    """Prepared local operator (init_bfun_main + primme_matvec, tt_eigb.f90:15-49).

    Binds torch CUDA tensors Phi1, A, Phi2; ``apply(X, Y, nvec)`` runs
    asynchronously on the context's stream (bound to torch's current stream).
    """

    def __init__(self, rx1, m, rx2, ry1, n, ry2, ra1, ra2, phi1, A, phi2, nvec_max=8,
                 method="plain", ctx=None):
        self._h = C.c_void_p()
        dims = (rx1, m, rx2, ry1, n, ry2, ra1, ra2)
        self._xy = (rx1 * m * rx2, ry1 * n * ry2)
        ptrs = (_dev(phi1, ry1 * rx1 * ra1, "float64", "phi1"),
                _dev(A, ra1 * n * m * ra2, "float64", "A"),
                _dev(phi2, rx2 * ra2 * ry2, "float64", "phi2"))
        self.ctx = _kctx(ctx)
        self._keep = (phi1, A, phi2)
        self.ctx.check(lib().ttg_localop_create(
            self.ctx.handle, *_dims(*dims), *ptrs, _i64(nvec_max), C.c_int(METHOD[method]),
            C.byref(self._h)))

    def apply(self, X, Y, nvec=1):
        nx, ny = self._xy
        self.ctx.check(lib().ttg_localop_apply(self._h, _dev(X, nx * nvec, "float64", "X"),
                                               _dev(Y, ny * nvec, "float64", "Y"), _i64(nvec)))

    def close(self):
        if self._h:
            lib().ttg_localop_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------- learned preconditioner
class LearnedPrec:
    """The learned preconditioner network of the plain local eigensolver (no
    counterpart in the reference, whose PRIMME preconditioner hook is unset,
    tt_eigb.f90:252-283).  ``widths`` = [3] + [width] * depth + [1]."""

    def __init__(self, width=512, depth=3, seed=0, ctx=None):
        self.ctx = ctx or default_context()
        self.width, self.depth = width, depth
        self._h = C.c_void_p()
        self.ctx.check(lib().ttg_mlp_create(self.ctx.handle, _i64(width), _i64(depth), _i64(seed),
                                            C.byref(self._h)))

    @property
    def handle(self):
        return self._h

    def nparams(self):
        return int(lib().ttg_mlp_nparams(self._h))

    def get_params(self):
        out = np.empty(self.nparams(), dtype=np.float32)
        self.ctx.check(lib().ttg_mlp_get_params(self._h, _p(out), _i64(len(out))))
        return out

    def set_params(self, flat):
        flat = np.ascontiguousarray(flat, dtype=np.float32)
        self.ctx.check(lib().ttg_mlp_set_params(self._h, _p(flat), _i64(len(flat))))

    def get_grads(self):
        out = np.empty(self.nparams(), dtype=np.float32)
        self.ctx.check(lib().ttg_mlp_get_grads(self._h, _p(out), _i64(len(out))))
        return out

    def forward(self, P, F, h):
        self.ctx.bind_torch_stream()
        self.ctx.check(lib().ttg_mlp_forward(self._h, _i64(P), _dev(F), _dev(h)))

    def loss_grad(self, N, B, D, theta, X, R, V):
        self.ctx.bind_torch_stream()
        loss = C.c_double()
        self.ctx.check(lib().ttg_mlp_loss_grad(self._h, _i64(N), _i64(B), _dev(D), _dev(theta),
                                               _dev(X), _dev(R), _dev(V), C.byref(loss)))
        return loss.value

    def adam_step(self, lr):
        self.ctx.check(lib().ttg_mlp_adam_step(self._h, C.c_double(lr)))

    def set_precision(self, bf16=True):
        """Layer products in BF16 on the tensor cores (default) or FP32."""
        self.ctx.check(lib().ttg_mlp_set_precision(self._h, C.c_int(1 if bf16 else 0)))

    def check(self):
        """Raise if a tensor-core product of the network gave up waiting."""
        self.ctx.check(lib().ttg_mlp_check(self._h))

    def train_recorded(self, rec_ctx, steps, lr=1e-4, seed=0):
        l0, l1 = C.c_double(), C.c_double()
        self.ctx.check(lib().ttg_mlp_train_recorded(self._h, rec_ctx.handle, _i64(steps),
                                                    C.c_double(lr), _i64(seed), C.byref(l0),
                                                    C.byref(l1)))
        return l0.value, l1.value

    def close(self):
        if self._h:
            lib().ttg_mlp_destroy(self._h)
            self._h = C.c_void_p()


def set_learned(mlp, mode, ctx=None):
    """mode bit 0: precondition the plain method's Davidson expansions with
    ``mlp``; bit 1: record the plain method's iterative local problems."""
    ctx = ctx or default_context()
    ctx.check(lib().ttg_set_learned(ctx.handle, mlp.handle if mlp is not None else C.c_void_p(),
                                    C.c_int(mode)))


def record_count(ctx=None):
    ctx = ctx or default_context()
    a, b = _i64(), _i64()
    ctx.check(lib().ttg_record_count(ctx.handle, C.byref(a), C.byref(b)))
    return a.value, b.value


def record_clear(ctx=None):
    ctx = ctx or default_context()
    ctx.check(lib().ttg_record_clear(ctx.handle))


# ---------------------------------------------------------- batched chains
class EigbBatch:
    """Many independent tt_eigb chains solved together (no counterpart in
    the reference): ``add`` queues a chain (inputs are copied), ``run``
    solves every queued chain on ``nworkers`` host threads with one stream
    each, ``result(i)`` returns (lambda, cores, ry, stats) like ``tt_eigb``."""

    def __init__(self, nworkers=8, ctx=None):
        self.ctx = ctx or default_context()
        self._h = C.c_void_p()
        self.ctx.check(lib().ttg_batch_create(self.ctx.handle, C.c_int(nworkers), C.byref(self._h)))
        self._meta = []

    def add(self, d, n, m, ra, crA, crY0, ry, eps, rmax, B, nswp=20, max_full_size=2000,
            method="plain"):
        n_, m_, ra_, ry_ = _iarr(n), _iarr(m), _iarr(ra), _iarr(ry)
        A_, Y_ = _darr(crA), _darr(crY0)
        _check_sizes("EigbBatch.add", d, {"n": n_, "m": m_}, {"ra": ra_, "ry": ry_},
                     [("crA", A_, ra_, n_, m_), ("crY0", Y_, ry_, n_)])
        idx = _i64()
        self.ctx.check(lib().ttg_batch_add_eigb(self._h, _i64(d), _p(n_), _p(m_), _p(ra_), _p(A_),
                                                _p(Y_), _p(ry_), C.c_double(eps), _i64(rmax),
                                                _i64(B), _i64(nswp), _i64(max_full_size),
                                                C.c_int(METHOD[method]), C.byref(idx)))
        self._meta.append((d, B))
        return idx.value

    def run(self):
        self.ctx.check(lib().ttg_batch_run(self._h))

    def result(self, i):
        d, B = self._meta[i]
        lam = np.zeros(B)
        ry = np.zeros(d + 1, dtype=np.int64)
        nc, mv = _i64(), _i64()
        sec = C.c_double()
        st = C.c_int()
        self.ctx.check(lib().ttg_batch_result(self._h, _i64(i), _p(lam), _p(ry), C.byref(nc),
                                              C.byref(mv), C.byref(sec), C.byref(st)))
        if st.value != TTG_OK:
            raise TTGError(st.value, f"batch chain {i} did not succeed")
        cores = np.zeros(nc.value)
        self.ctx.check(lib().ttg_batch_cores(self._h, _i64(i), _p(cores), _i64(nc.value)))
        return lam, cores, [int(v) for v in ry], {"matvecs": mv.value, "seconds": sec.value}

    def close(self):
        if self._h:
            lib().ttg_batch_destroy(self._h)
            self._h = C.c_void_p()
