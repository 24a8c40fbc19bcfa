"""The allocation-free L2-norm entry point, through the C ABI.

nrgpu_l2_norm_sq_static serves callers that cannot allocate device memory
(host codes that own all device memory and forbid allocation in their time
loop, or C/Fortran drivers without a device allocator): its partial sums live
in a fixed array inside the library instead of caller scratch.  Both entry
points launch the same reduction with the same block count, so their results
must agree bit for bit.  The calls run on a large grid first (the block count
at its SM-count cap, so the fixed array holds many partials) and then on a
small one, two calls on each, so a stale partial left by an earlier call
would show.  It sits in a file pytest collects last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims_seq", [((128, 128, 64), (40, 24, 16))])
def test_static_scratch_l2_matches_allocating_entry_point(cuda, dims_seq):
    import torch
    from nrpytutorial_gb300 import Grid, _lib
    lib = _lib.load()
    _lib.set_stream(torch.cuda.current_stream())
    scratch = torch.zeros(4096, dtype=torch.float64, device=cuda)
    rng = np.random.default_rng(2024)
    for dims in dims_seq:
        G = Grid("Cartesian", dims, FD_order=4, NGHOSTS=2)
        f = torch.tensor(rng.standard_normal((2,) + G.shape), device=cuda)
        p = C.byref(G.params)
        for gf in (0, 1):  # two calls in a row, different data each time
            want = torch.zeros(2, dtype=torch.float64, device=cuda)
            got = torch.zeros(2, dtype=torch.float64, device=cuda)
            _lib.check(lib.nrgpu_l2_norm_sq(p, _lib.ptr(f), gf, _lib.ptr(scratch), 4096, _lib.ptr(want)),
                       "nrgpu_l2_norm_sq")
            _lib.check(lib.nrgpu_l2_norm_sq_static(p, _lib.ptr(f), gf, _lib.ptr(got)), "nrgpu_l2_norm_sq_static")
            torch.cuda.synchronize()
            w, g = want.tolist(), got.tolist()
            assert g[1] == w[1] == dims[0] * dims[1] * dims[2]
            assert g[0] == w[0], (dims, gf, g, w)
            # and the value itself: the sum of squares over the interior
            ng = 2
            ref = float((f[gf, ng:-ng, ng:-ng, ng:-ng] ** 2).sum())
            assert abs(g[0] - ref) <= 1e-12 * ref
