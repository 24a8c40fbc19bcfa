"""The allocation-free L2-norm entry point, through the C ABI.

nrgpu_l2_norm_sq_static serves callers that cannot allocate device memory
(host codes that own all device memory and forbid allocation in their time
loop, or C/Fortran drivers without a device allocator): its partial sums live
in a fixed array inside the library instead of caller scratch.  This test
checks that two calls in a row, on different data, agree with the allocating
entry point nrgpu_l2_norm_sq within the tolerance the other reduction tests
use.  It sits in a file pytest collects last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def test_static_scratch_l2_matches_allocating_entry_point(cuda):
    import torch
    from nrpytutorial_gb300 import Grid, _lib
    lib = _lib.load()
    G = Grid("Cartesian", (40, 24, 16), FD_order=4, NGHOSTS=2)
    rng = np.random.default_rng(2024)
    f = torch.tensor(rng.standard_normal((2,) + G.shape), device=cuda)
    _lib.set_stream(torch.cuda.current_stream())
    scratch = torch.zeros(4096, dtype=torch.float64, device=cuda)
    want = torch.zeros(2, dtype=torch.float64, device=cuda)
    got = torch.zeros(2, dtype=torch.float64, device=cuda)
    p = C.byref(G.params)
    for gf in (0, 1):  # two calls in a row, different data each time
        _lib.check(lib.nrgpu_l2_norm_sq(p, _lib.ptr(f), gf, _lib.ptr(scratch), 4096, _lib.ptr(want)),
                   "nrgpu_l2_norm_sq")
        _lib.check(lib.nrgpu_l2_norm_sq_static(p, _lib.ptr(f), gf, _lib.ptr(got)), "nrgpu_l2_norm_sq_static")
        torch.cuda.synchronize()
        w, g = want.tolist(), got.tolist()
        assert g[1] == w[1] == 40 * 24 * 16
        assert abs(g[0] - w[0]) <= TOL * abs(w[0]), (gf, g, w)
