"""Curvilinear boundary conditions on the GPU vs the oracle: the flattened
ghost-zone map (integer-exact) and its application (bit-exact in FP64,
since both evaluate 3 f1 - 3 f2 + f3 left to right without contraction)."""
import numpy as np
import pytest

import oracle.bcs as ob
from tests.helpers import grids

pytestmark = pytest.mark.gpu

CASES = [("Spherical", (4, 4, 4), 3), ("SinhSpherical", (8, 6, 4), 3), ("Cartesian", (6, 5, 7), 2),
         ("Spherical", (6, 4, 8), 2), ("SinhSpherical", (10, 8, 6), 4), ("SinhSphericalv2", (10, 8, 6), 3),
         ("Cylindrical", (6, 6, 6), 3), ("SinhCylindrical", (8, 6, 8), 3), ("SinhCylindricalv2", (8, 6, 8), 3),
         ("SymTP", (8, 6, 4), 3), ("SinhSymTP", (8, 6, 8), 3)]


@pytest.mark.parametrize("coord,Nxx,ng", CASES)
def test_bc_map_matches_oracle(cuda, coord, Nxx, ng):
    from nrpytutorial_gb300 import Evolution
    G, gp = grids("BSSN", coord, Nxx, 4, ng=ng)
    ev = Evolution("BSSN", G, device=cuda)
    m = ev.bc_map()
    layers = ob.build_bcstruct(gp)
    od, os_, idst, isrc, ipar = [], [], [], [], []
    for g, (outer, (d, s, p)) in enumerate(layers):
        start = len(od)
        assert m["ob_dir_start"][g][0] == start
        for k, arr in enumerate(outer):
            od += list(arr[:, 0])
            os_ += list(arr[:, 1])
            assert m["ob_dir_start"][g][k + 1] == len(od)
        assert m["num_ob"][g] == len(od) - start
        assert m["ib_start"][g] == len(idst)
        assert m["num_ib"][g] == len(d)
        idst += list(d)
        isrc += list(s)
        ipar += [int(sum((1 << t) for t in range(10) if row[t] < 0)) for row in p]
    assert np.array_equal(m["outer_dest"], od)
    assert np.array_equal(m["outer_step"], os_)
    assert np.array_equal(m["inner_dest"], idst)
    assert np.array_equal(m["inner_src"], isrc)
    assert np.array_equal(m["inner_parity"], ipar)


@pytest.mark.parametrize("coord,Nxx,ng", CASES)
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_apply_bcs_matches_oracle(cuda, coord, Nxx, ng, dtype):
    import torch
    from nrpytutorial_gb300 import Evolution, SYSTEM_GFS
    G, gp = grids("BSSN", coord, Nxx, 4, ng=ng)
    ev = Evolution("BSSN", G, device=cuda)
    parity = SYSTEM_GFS["BSSN"][1]
    f = np.random.default_rng(5).standard_normal((24,) + gp.shape).astype(dtype)
    t = torch.tensor(f, device=cuda)
    ev.apply_bcs(t)
    ref = ob.apply_bcs(ob.build_bcstruct(gp), f.copy(), parity)
    assert np.array_equal(t.cpu().numpy(), ref)
