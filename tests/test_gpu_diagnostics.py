"""Constraint diagnostics on the GPU: the interior L2-norm reduction (FP64
accumulation, deterministic two-pass with a caller-provided scratch array)
and the Maxwell divergence constraint vs the oracle."""
import ctypes as C

import numpy as np
import pytest

import oracle.wave_maxwell as ow
from tests.helpers import grids, per_gf_rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nblk", [1, 7, 1024])
def test_l2_norm_matches_numpy(cuda, nblk):
    import torch
    from nrpytutorial_gb300 import Evolution, _lib
    G, gp = grids("ScalarWave", "Cartesian", (30, 20, 10), 4)
    ev = Evolution("ScalarWave", G, device=cuda)
    f = np.random.default_rng(4).standard_normal((2,) + gp.shape)
    t = torch.tensor(f, device=cuda)
    scratch = torch.zeros(nblk, dtype=torch.float64, device=cuda)
    res = torch.zeros(2, dtype=torch.float64, device=cuda)
    for gf in (0, 1):
        _lib.check(ev.lib.nrgpu_l2_norm_sq(C.byref(G.params), _lib.ptr(t), gf, _lib.ptr(scratch), nblk,
                                           _lib.ptr(res)), "l2")
        s, n = res.tolist()
        want = (gp.interior(f[gf]) ** 2).sum()
        assert n == 30 * 20 * 10
        assert abs(s - want) <= 1e-12 * want
    # deterministic: the same call gives the same bits
    _lib.check(ev.lib.nrgpu_l2_norm_sq(C.byref(G.params), _lib.ptr(t), 1, _lib.ptr(scratch), nblk,
                                       _lib.ptr(res)), "l2")
    a = res.clone()
    _lib.check(ev.lib.nrgpu_l2_norm_sq(C.byref(G.params), _lib.ptr(t), 1, _lib.ptr(scratch), nblk,
                                       _lib.ptr(res)), "l2")
    assert torch.equal(a, res)


def test_maxwell_constraint_matches_oracle(cuda):
    import torch
    from nrpytutorial_gb300 import Evolution
    G, gp = grids("Maxwell", "Cartesian", (12, 12, 12), 4)
    ev = Evolution("Maxwell", G, device=cuda)
    f = ow.toroidal_dipole(gp, 0.3)
    Cc = ev.maxwell_constraint(torch.tensor(f, device=cuda)).cpu().numpy()
    ref = ow.maxwell_constraint_grid(gp, f)
    g = gp.NGHOSTS
    assert per_gf_rel(Cc[:, g:-g, g:-g, g:-g], ref[None, g:-g, g:-g, g:-g]) < 1e-12
