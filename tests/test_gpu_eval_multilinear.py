"""GPU tests of gkrgpu_eval_multilinear against the oracle's eval_multilinear
(include/poly_commit/poly.hpp:88-104).  Exact: tolerance zero."""
import numpy as np
import pytest

from gkr_gb300 import circuit as gc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nb_vars,n,points", [(0, 4, 1), (1, 8, 2), (5, 16, 3), (10, 48, 3), (12, 1024, 2),
                                              (16, 64, 3)])
def test_eval_multilinear_matches_oracle(ctx, oracle, nb_vars, n, points):
    from gkr_gb300.prover import DeviceBuffer
    st = gc.Stream(nb_vars * 1000 + n)
    table = st.field((1 << nb_vars) * n).reshape(1 << nb_vars, n)
    pts = st.field(points * nb_vars).reshape(points, nb_vars)
    d = DeviceBuffer(ctx, table.nbytes)
    d.upload(table)
    got = ctx.eval_multilinear(d.ptr, nb_vars, n, pts)
    for j in range(points):
        assert np.array_equal(got[j], oracle.eval_multilinear(table, pts[j]))
    # the reduction scratch is left clean: a second call gives the same answer
    assert np.array_equal(ctx.eval_multilinear(d.ptr, nb_vars, n, pts), got)


def test_eval_multilinear_rejects_bad_arguments(ctx):
    from gkr_gb300._lib import GkrGpuError
    from gkr_gb300.prover import DeviceBuffer
    d = DeviceBuffer(ctx, 16 * 16 * 4)
    with pytest.raises(GkrGpuError):
        ctx.eval_multilinear(d.ptr, 4, 16, np.zeros((4, 4), np.uint32))  # 4 points
    with pytest.raises(GkrGpuError):
        ctx.eval_multilinear(d.ptr, 4, 16, np.full((1, 4), gc.P, np.uint32))  # non-canonical point
