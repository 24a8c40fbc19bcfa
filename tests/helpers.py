"""Shared helpers for the parity tests: seeded fields, error norms, and the
paired (GPU grid, oracle grid) construction."""
import numpy as np

import oracle.grid as og

SEED = 20251203


def rel_l2(a, b):
    """Normwise relative error ||a-b||_2 / ||b||_2 (|| ||_2 over all entries)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (nb if nb > 0 else 1.0))


def per_gf_rel(a, b, ng=None):
    """Max over gridfunctions of the normwise relative error (interior if ng)."""
    worst = 0.0
    for g in range(a.shape[0]):
        x, y = a[g], b[g]
        if ng:
            x = x[ng:-ng, ng:-ng, ng:-ng]
            y = y[ng:-ng, ng:-ng, ng:-ng]
        worst = max(worst, rel_l2(x, y))
    return worst


def grids(system, coord, Nxx, fd_order, ng=None, **kw):
    """Matching product Grid and oracle GridParams."""
    from nrpytutorial_gb300 import Grid, default_nghosts
    ng = ng if ng is not None else default_nghosts(system, fd_order)
    G = Grid(coord, Nxx, FD_order=fd_order, NGHOSTS=ng, **kw)
    okw = {k: v for k, v in kw.items() if k in ("AMPL", "SINHW", "RMAX", "domain", "eta", "wavespeed", "const_dr",
                                                "bScale", "SINHWAA", "AMAX")}
    gp = og.GridParams(coord, Nxx, ng, fd_order, **okw)
    return G, gp


def bssn_random_state(shape, seed=SEED, amp=0.1):
    """24 BSSN gridfunctions: flat space plus seeded perturbations, so gammabar
    stays positive definite and cf, alpha stay positive."""
    rng = np.random.default_rng(seed)
    f = amp * (2 * rng.random((24,) + tuple(shape)) - 1)
    from oracle.bssn import GF
    f[GF["cf"]] += 1.0
    f[GF["alpha"]] += 1.0
    return f


def smooth_state(ngf, gp, seed=SEED, amp=0.1, offsets=None):
    """Sum of low-wavenumber sines of the grid indices, seeded."""
    rng = np.random.default_rng(seed)
    n2, n1, n0 = gp.shape
    i2, i1, i0 = np.meshgrid(np.arange(n2), np.arange(n1), np.arange(n0), indexing="ij")
    out = np.zeros((ngf,) + gp.shape)
    for g in range(ngf):
        for _ in range(3):
            k = rng.uniform(0.05, 0.4, 3)
            ph = rng.uniform(0, 2 * np.pi)
            out[g] += amp / 3 * np.sin(k[0] * i0 + k[1] * i1 + k[2] * i2 + ph)
    if offsets is not None:
        for g, o in offsets.items():
            out[g] += o
    return out


# Sommerfeld fixture configurations (tests/golden/ref_sommerfeld.npz): name ->
# (CoordSystem, d_r FD order); ScalarWave, FD4, 2 ghosts, on this grid.
SOMMERFELD_CFGS = {"somm_sph_dr2": ("Spherical", 2), "somm_sph_dr4": ("Spherical", 4),
                   "somm_sinhsph_dr2": ("SinhSpherical", 2), "somm_sinhsph_dr4": ("SinhSpherical", 4)}
SOMMERFELD_GRID = dict(Nxx=(10, 8, 6), AMPL=5.0, SINHW=0.3, RMAX=5.0)


def sommerfeld_inputs(coord_dr, shape):
    """Seeded (gfs, rhs) of a Sommerfeld fixture configuration."""
    coord, dr = coord_dr
    rng = np.random.default_rng(dr + 100 * (coord == "SinhSpherical"))
    return rng.standard_normal((2,) + shape), rng.standard_normal((2,) + shape)
