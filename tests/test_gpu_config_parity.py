"""FP64 parity at the benchmark configurations' own grid sizes, against the
reference's generated C (strict FP64 build in oracle/_ref, compiled on this
machine by __graft_entry__.build() from the output of oracle/gen_ref.py):

* the BSSN SinhSpherical headline grid -- 128 x 64 x 16 interior, AMPL 64,
  SINHW 0.2, FD4, 3 ghosts -- with Brill-Lindquist data (m = 0.5 at
  z = +-0.5) plus a seeded smooth perturbation;
* a z-slab of the BSSN Cartesian 256^3 FD6 configuration -- the full
  256 x 256 extent in i0, i1 at its grid spacing (20/256 on [-10, 10]),
  8 planes in i2, 4 ghosts -- with its seeded Brill-Lindquist data plus a
  perturbation.

Ricci_eval and the det(gammabar) rescale must match at 1e-12 normwise
relative per gridfunction; rhs_eval (given the reference's RbarDD) and
the Hamiltonian constraint at 1e-11; with every BSSN kernel family.  The
identical FP64 input state goes to both sides.  The 1e-11 bounds are the
FP64 conditioning of these sums of large cancelling terms at
Brill-Lindquist data, not a kernel property: on the same kind of input the
numpy oracle, an independent FP64 evaluation, differs from the reference's
C by up to 3e-12 per gridfunction in the RHS (aDD_ii and trK; a 64 x 64 x 8
Cartesian FD6 slab at this grid spacing) and by 5.4e-12 (64 x 64 x 8
Cartesian FD6) and 1.3e-12 (64 x 32 x 16 SinhSpherical FD4) in H; the GPU's
point, staged and fused kernels show the same figures as each other (RHS
5e-12 on the 256^2 x 8 slab and 1.5e-12 on the headline grid; H 3.9e-12
and 1.2e-12).  The rescale acts on gammabar ~ 1 while hDD is ~1e-3 here,
so FP64 rounding of gammabar is ~1e-13 relative to hDD: oracle vs the
reference's C 4.0e-13 (Cartesian FD6 slab) and 5.0e-13 (SinhSpherical),
GPU 5.0e-13 and 4.8e-13.
"""
import numpy as np
import pytest

import oracle.grid as og
from oracle import ref
from tests.helpers import per_gf_rel, smooth_state

pytestmark = pytest.mark.gpu

TOL = 1e-12
RHS_TOL = 1e-11


def _reference(cfg, gp):
    if not ref.available(cfg):
        pytest.skip("reference-generated C %s not built on this machine (oracle/gen_ref.py output absent)" % cfg)
    return ref.RefKernels(cfg, gp)


def _compare(cuda, G, gp, cfg, m1, z1, m2, z2, seed):
    import torch
    from nrpytutorial_gb300 import Evolution
    ev = Evolution("BSSN", G, precision="fp64", device=cuda)
    ev.initial_data_brill_lindquist(m1, (0.0, 0.0, z1), m2, (0.0, 0.0, z2))
    ev.apply_bcs(ev.y_n)
    ev.enforce_detgammabar(ev.y_n)
    f = ev.y_n.cpu().numpy() + smooth_state(24, gp, seed=seed, amp=1e-3)
    f = np.ascontiguousarray(f)
    rk = _reference(cfg, gp)
    t = torch.tensor(f, device=cuda)
    g = gp.NGHOSTS
    interior = (slice(None), slice(g, -g), slice(g, -g), slice(g, -g))

    aux = torch.zeros((6,) + gp.shape, dtype=torch.float64, device=cuda)
    ev.ricci_eval(t, aux)
    r_ric = rk.ricci(f)
    assert per_gf_rel(aux.cpu().numpy()[interior], r_ric[interior]) < TOL

    out = torch.zeros_like(t)
    ev.rhs_eval_given_ricci(t, torch.tensor(r_ric, device=cuda), out)
    r_rhs = rk.rhs_eval(f, aux=r_ric)
    assert per_gf_rel(out.cpu().numpy()[interior], r_rhs[interior]) < RHS_TOL

    H = ev.hamiltonian(t).cpu().numpy()[0]
    r_H = rk.hamiltonian(f)
    assert per_gf_rel(H[None, g:-g, g:-g, g:-g], r_H[None, g:-g, g:-g, g:-g]) < RHS_TOL

    t2 = t.clone()
    ev.enforce_detgammabar(t2)
    r_enf = rk.enforce(f)
    assert per_gf_rel(t2.cpu().numpy()[11:17], r_enf[11:17]) < TOL


def test_headline_grid_matches_reference_generated_c(cuda, bssn_kernels):
    from nrpytutorial_gb300 import Grid
    kw = dict(AMPL=64.0, SINHW=0.2, eta=2.0)
    G = Grid("SinhSpherical", (128, 64, 16), FD_order=4, NGHOSTS=3, **kw)
    gp = og.GridParams("SinhSpherical", (128, 64, 16), 3, 4, **kw)
    _compare(cuda, G, gp, "bssn_sinhsph_fd4", 0.5, 0.5, 0.5, -0.5, seed=41)


def test_cartesian_256_fd6_slab_matches_reference_generated_c(cuda, bssn_kernels):
    from nrpytutorial_gb300 import Grid
    rng = np.random.default_rng(3)  # the configuration's own seeded masses and positions
    m1, m2 = rng.uniform(0.3, 0.7, 2)
    z1, z2 = rng.uniform(0.3, 1.0), -rng.uniform(0.3, 1.0)
    dz = 20.0 / 256
    dom = ((-10.0, 10.0), (-10.0, 10.0), (-4 * dz, 4 * dz))
    G = Grid("Cartesian", (256, 256, 8), FD_order=6, NGHOSTS=4, domain=dom, eta=2.0)
    gp = og.GridParams("Cartesian", (256, 256, 8), 4, 6, domain=dom, eta=2.0)
    assert np.allclose(gp.dxx, [dz] * 3)
    _compare(cuda, G, gp, "bssn_cart_fd6", m1, z1, m2, z2, seed=43)
