"""The reference's C caller links against the library unchanged (CPU).

gmres_3d.c (tt-fort's C GMRES for the local AMEn system) declares dbfun3 and
djac_apply with by-reference `long*` arguments (gmres_3d.c:3-4) and calls the
BLAS with 64-bit integers.  oracle/build_ref.py compiles it unchanged from the
tt-fort source tree and links it against libttgpu.so with every symbol
resolved: dbfun3 and djac_apply come from the library, the BLAS from the
oracle's forwarder.  Skipped without the source tree; the numerics of the
same calls are checked on the GPU in test_fshim_gpu.py."""
import ctypes as C

import pytest

from oracle import build_ref


@pytest.mark.skipif(build_ref.source_tree() is None, reason="tt-fort source tree absent")
def test_gmres_3d_links_against_library():
    import ttgpu
    path = build_ref.build_gmres3d(ttgpu.LIB_PATH)
    lib = C.CDLL(path)
    for name in ("dgmresr_hh", "dgmresl_hh", "dgmresr_hh_", "dgmresl_hh_"):
        assert hasattr(lib, name)
    # dbfun3 / djac_apply in the linked object resolve to libttgpu.so
    tt = ttgpu.lib()
    for name in ("dbfun3", "djac_apply", "djac_gen", "dqr"):
        assert hasattr(tt, name)
