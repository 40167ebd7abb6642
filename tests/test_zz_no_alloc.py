"""GPU test of gkrgpu_eval_multilinear_noalloc, the entry point for callers that cannot
allocate device memory (for example a verifier inside a process whose device memory is
already held by another framework's caching allocator, or code that must not call
cudaMalloc/cudaFree because they can synchronize the device).

It is called through the C ABI and compared with the allocating gkrgpu_eval_multilinear
on the same table and points, exactly (integer field results, tolerance zero), on two
calls in a row, so that a scratch region left dirty by the first call would show up in
the second.  This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from gkr_gb300 import circuit as gc

pytestmark = pytest.mark.gpu


# 1028, 2044 and 4084 copies: n_copies / 4 has no divisor between 2 and 32 (257 is prime,
# 511 = 7 x 73, 1021 is prime, so row slices of 4 or 28 copies), giving 257, 73 and 1021
# lane groups, each with its own arrival ticket in the fixed scratch.
@pytest.mark.parametrize("nb_vars,n,points", [(18, 64, 3), (12, 4096, 2), (6, 4, 1), (0, 8, 3),
                                              (10, 1028, 3), (9, 2044, 2), (8, 4084, 1)])
def test_noalloc_matches_allocating_entry_point(ctx, nb_vars, n, points):
    from gkr_gb300 import _lib
    from gkr_gb300.prover import DeviceBuffer
    lib = _lib.load()
    st = gc.Stream(77 + nb_vars * 131 + n)
    table = st.field((1 << nb_vars) * n).reshape(1 << nb_vars, n)
    d_in = DeviceBuffer(ctx, table.nbytes)
    d_in.upload(table)
    d_out = DeviceBuffer(ctx, points * n * 4)
    for call in range(2):
        pts = st.field(points * nb_vars).reshape(points, nb_vars)
        want = ctx.eval_multilinear(d_in.ptr, nb_vars, n, pts)
        rc = lib.gkrgpu_eval_multilinear_noalloc(ctypes.c_void_p(d_in.ptr), nb_vars, n, pts.ctypes.data, points,
                                                 ctypes.c_void_p(d_out.ptr), None)
        assert rc == 0, lib.gkrgpu_last_error()
        got = np.empty((points, n), np.uint32)
        _lib.check(lib.gkrgpu_memcpy_d2h(ctx.handle, got.ctypes.data, ctypes.c_void_p(d_out.ptr), got.nbytes))
        assert np.array_equal(got, want), f"call {call}"


def test_noalloc_rejects_sizes_beyond_its_scratch(ctx):
    from gkr_gb300 import _lib
    from gkr_gb300.prover import DeviceBuffer
    lib = _lib.load()
    d = DeviceBuffer(ctx, 4096)
    pts = np.zeros((1, 19), np.uint32)
    assert lib.gkrgpu_eval_multilinear_noalloc(ctypes.c_void_p(d.ptr), 19, 4, pts.ctypes.data, 1,
                                               ctypes.c_void_p(d.ptr), None) == _lib.ERR_INVALID
    assert b"18" in lib.gkrgpu_last_error()
    pts = np.zeros((1, 2), np.uint32)
    assert lib.gkrgpu_eval_multilinear_noalloc(ctypes.c_void_p(d.ptr), 2, 8192, pts.ctypes.data, 1,
                                               ctypes.c_void_p(d.ptr), None) == _lib.ERR_INVALID
