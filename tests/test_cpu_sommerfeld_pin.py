"""The oracle's Sommerfeld restatement (oracle/bcs.py apply_sommerfeld)
against the reference's own generated apply_bcs_sommerfeld
(CurviBoundaryConditions.py:259-658 via oracle/gen_ref_somm.py; fixture
tests/golden/ref_sommerfeld.npz): ScalarWave on Spherical and SinhSpherical
grids at d_r FD orders 2 and 4, the RHS at every point after the boundary
condition, to roundoff."""
import os

import numpy as np
import pytest

import oracle.bcs as ob
import oracle.grid as og
from tests.helpers import SOMMERFELD_CFGS, SOMMERFELD_GRID, sommerfeld_inputs

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("cfg", sorted(SOMMERFELD_CFGS))
def test_oracle_sommerfeld_matches_reference_generated_c(cfg):
    coord, dr = SOMMERFELD_CFGS[cfg]
    g = SOMMERFELD_GRID
    gp = og.GridParams(coord, g["Nxx"], 2, 4, AMPL=g["AMPL"], SINHW=g["SINHW"], RMAX=g["RMAX"])
    f, rhs = sommerfeld_inputs(SOMMERFELD_CFGS[cfg], gp.shape)
    want = np.load(os.path.join(GOLD, "ref_sommerfeld.npz"))[cfg]
    assert np.any(want != rhs)
    got = ob.apply_sommerfeld(gp, ob.build_bcstruct(gp), f, rhs.copy(), [0, 0], dr)
    assert np.abs(got - want).max() <= 1e-15 * np.abs(want).max() * 10
