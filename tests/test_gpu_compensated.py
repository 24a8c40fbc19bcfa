"""Compensated mixed precision (NRGPU_PREC_COMPENSATED): FP32 RHS arithmetic
on split FP32 stage inputs (hi + remainder), FP64 y_n and running total.
Against the FP64 step it must be far closer than the plain FP32-stage mode,
fused and unfused steps must agree, and graph replay must match eager steps.
The same for NRGPU_PREC_COMPENSATED_FP64RK, whose RK accumulation and
det(gammabar) rescale are FP64 arithmetic: its error against FP64 is that of
the FP32 RHS alone."""
import numpy as np
import pytest

from tests.helpers import grids, rel_l2, smooth_state

pytestmark = pytest.mark.gpu

KW = dict(AMPL=5.0, SINHW=0.3, RMAX=5.0, domain=(-2.0, 2.0), eta=2.0)


def _evo(cuda, system, coord, Nxx, order, prec):
    from nrpytutorial_gb300 import Evolution
    G, gp = grids(system, coord, Nxx, order, **KW)
    return Evolution(system, G, precision=prec, device=cuda), gp


def _state(system, gp):
    if system == "ScalarWave":
        return smooth_state(2, gp, seed=1, amp=1.0, offsets={0: 2.0})
    if system == "Maxwell":
        return smooth_state(7, gp, seed=2, amp=1.0, offsets={3: 1.5})
    from oracle.bssn import GF
    return smooth_state(24, gp, seed=3, amp=0.05, offsets={GF["alpha"]: 1.0, GF["cf"]: 1.0})


def _run(cuda, system, coord, Nxx, order, prec, y, dt, n, fused=True):
    import torch
    ev, gp = _evo(cuda, system, coord, Nxx, order, prec)
    ev.y_n.copy_(torch.tensor(y, device=cuda))
    ev.apply_bcs(ev.y_n)
    if system == "BSSN":
        ev.enforce_detgammabar(ev.y_n)
    for _ in range(n):
        ev.step(dt, fused=fused)
    torch.cuda.synchronize()
    return ev.y_n.cpu().numpy()


CASES = [("ScalarWave", "SinhSpherical", (16, 12, 8), 4),
         ("ScalarWave", "Cartesian", (16, 16, 16), 4),
         ("Maxwell", "Cartesian", (16, 16, 16), 4),
         ("BSSN", "Cartesian", (12, 12, 12), 4),
         ("BSSN", "SinhSpherical", (12, 10, 8), 4),
         ("BSSN", "SinhSphericalv2", (12, 10, 8), 4),
         ("BSSN", "SinhCylindrical", (12, 10, 8), 4),
         ("BSSN", "SinhSymTP", (12, 10, 8), 4)]


@pytest.mark.parametrize("system,coord,Nxx,order", CASES)
def test_compensated_much_closer_to_fp64_than_plain_fp32(cuda, system, coord, Nxx, order):
    from nrpytutorial_gb300 import default_nghosts
    G, gp = grids(system, coord, Nxx, order, **KW)
    y = _state(system, gp)
    dt = G.find_timestep(0.5)
    n = 8
    ref = _run(cuda, system, coord, Nxx, order, "fp64", y, dt, n)
    plain = _run(cuda, system, coord, Nxx, order, "mixed", y, dt, n)
    comp = _run(cuda, system, coord, Nxx, order, "compensated", y, dt, n)
    g = default_nghosts(system, order)
    sl = (slice(None), slice(g, -g), slice(g, -g), slice(g, -g))
    e_plain = rel_l2(plain[sl], ref[sl])
    e_comp = rel_l2(comp[sl], ref[sl])
    print("%s %s: state rel_l2 plain %.3e compensated %.3e" % (system, coord, e_plain, e_comp))
    # measured on GB300: 20-300x smaller than plain FP32 stages (4x for the
    # poorly resolved Maxwell noise, where FP32 arithmetic dominates)
    assert e_comp < 1e-6, e_comp
    assert e_comp < e_plain / 3, (e_comp, e_plain)


@pytest.mark.parametrize("system,coord,Nxx,order", CASES)
def test_fp64_accumulation_form_close_to_fp64(cuda, system, coord, Nxx, order):
    """FP32 RHS with FP64 RK accumulation and FP64 rescale: the error against
    the FP64 step is the FP32 RHS's, at the float-float form's level."""
    from nrpytutorial_gb300 import default_nghosts
    G, gp = grids(system, coord, Nxx, order, **KW)
    y = _state(system, gp)
    dt = G.find_timestep(0.5)
    n = 8
    ref = _run(cuda, system, coord, Nxx, order, "fp64", y, dt, n)
    comp = _run(cuda, system, coord, Nxx, order, "compensated", y, dt, n)
    acc = _run(cuda, system, coord, Nxx, order, "compensated_fp64rk", y, dt, n)
    g = default_nghosts(system, order)
    sl = (slice(None), slice(g, -g), slice(g, -g), slice(g, -g))
    e_comp, e_acc = rel_l2(comp[sl], ref[sl]), rel_l2(acc[sl], ref[sl])
    print("%s %s: state rel_l2 compensated %.3e fp64-accumulation %.3e" % (system, coord, e_comp, e_acc))
    assert e_acc < 1e-6, e_acc
    assert e_acc < 2 * e_comp + 1e-14, (e_acc, e_comp)


@pytest.mark.parametrize("prec", ["compensated", "compensated_fp64rk"])
@pytest.mark.parametrize("system,coord,Nxx,order", [CASES[0], CASES[2], CASES[4]])
def test_compensated_fused_equals_unfused(cuda, system, coord, Nxx, order, prec):
    G, gp = grids(system, coord, Nxx, order, **KW)
    y = _state(system, gp)
    dt = G.find_timestep(0.5)
    a = _run(cuda, system, coord, Nxx, order, prec, y, dt, 3, fused=True)
    b = _run(cuda, system, coord, Nxx, order, prec, y, dt, 3, fused=False)
    if prec == "compensated":  # both forms apply ff_rk4_pairs to the same k
        assert np.array_equal(a, b)
    assert rel_l2(a, b) < 1e-13


@pytest.mark.parametrize("prec", ["compensated", "mixed", "compensated_fp64rk"])
@pytest.mark.parametrize("coord", ["SinhSpherical", "SinhSymTP", "Cartesian"])
def test_split_update_step_equals_the_unfused_step_bitwise(cuda, coord, prec):
    """BSSN with FP32 stages: the step's kernel stores k and a separate
    kernel updates the interior points (staged and fused kernels, in
    float-float or FP64 arithmetic; the point kernels with plain FP32
    stages), the arithmetic the unfused step applies at every point, so the
    states agree bit for bit."""
    import torch
    system, order = "BSSN", 4
    Nxx = (12, 12, 12) if coord == "Cartesian" else (12, 10, 8)
    G, gp = grids(system, coord, Nxx, order, **KW)
    y = _state(system, gp)
    dt = G.find_timestep(0.5)
    a = _run(cuda, system, coord, Nxx, order, prec, y, dt, 3, fused=True)
    b = _run(cuda, system, coord, Nxx, order, prec, y, dt, 3, fused=False)
    assert np.array_equal(a, b)
    ev, _ = _evo(cuda, system, coord, Nxx, order, prec)
    ev.y_n.copy_(torch.tensor(y, device=cuda))
    ev.step(dt)
    ev.substep_rhs(dt, 1, 4)  # the update kernel exists for this step


@pytest.mark.parametrize("prec", ["compensated", "mixed", "compensated_fp64rk"])
def test_substep_rhs_kernel_then_update_kernel_equals_the_substep(cuda, prec):
    """MoL_substep_rhs on a split step: the RHS kernel alone (which = 3) and
    then the update kernel alone (which = 4) leave every buffer as the whole
    substep (which = 0) does, byte for byte.  (A lone substep after a full
    step reads the FP64 y_n words as pairs, so some of its values are not
    finite; both forms produce the same words.)"""
    import torch
    system, coord, Nxx, order = "BSSN", "SinhSpherical", (12, 10, 8), 4
    G, gp = grids(system, coord, Nxx, order, **KW)
    y = _state(system, gp)
    dt = G.find_timestep(0.5)

    def run(whiches):
        ev, _ = _evo(cuda, system, coord, Nxx, order, prec)
        ev.y_n.copy_(torch.tensor(y, device=cuda))
        ev.apply_bcs(ev.y_n)
        ev.enforce_detgammabar(ev.y_n)
        ev.step(dt)
        for w in whiches:
            ev.substep_rhs(dt, 1, w)
        torch.cuda.synchronize()
        return [t.cpu().numpy().copy() for t in (ev.y_n, ev.rt, ev.k_odd, ev.k_even)]

    whole, parts = run([0]), run([3, 4])
    for a, b in zip(whole, parts):
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("prec", ["compensated", "compensated_fp64rk"])
def test_compensated_graph_replay_matches_eager(cuda, prec):
    import torch
    system, coord, Nxx, order = CASES[4]
    G, gp = grids(system, coord, Nxx, order, **KW)
    y = _state(system, gp)
    dt = G.find_timestep(0.5)
    eager = _run(cuda, system, coord, Nxx, order, prec, y, dt, 3)
    ev, _ = _evo(cuda, system, coord, Nxx, order, prec)
    ev.y_n.copy_(torch.tensor(y, device=cuda))
    ev.apply_bcs(ev.y_n)
    ev.enforce_detgammabar(ev.y_n)
    replay = ev.capture(dt, n_steps=3)
    replay()
    torch.cuda.synchronize()
    assert np.array_equal(ev.y_n.cpu().numpy(), eager)


def test_compensated_stage_buffers_are_pairs(cuda):
    """After a step the substep buffers hold (hi, lo) pairs: hi is the FP32
    rounding of hi + lo and |lo| is at most half an FP32 ulp of hi."""
    import torch
    system, coord, Nxx, order = CASES[0]
    G, gp = grids(system, coord, Nxx, order, **KW)
    ev, _ = _evo(cuda, system, coord, Nxx, order, "compensated")
    ev.y_n.copy_(torch.tensor(_state(system, gp), device=cuda))
    ev.step(G.find_timestep(0.5))
    torch.cuda.synchronize()
    k = ev.k_odd.cpu().numpy()
    hi, lo = k[..., 0].astype(np.float64), k[..., 1].astype(np.float64)
    assert np.array_equal((hi + lo).astype(np.float32).astype(np.float64), hi)
    assert np.all(np.abs(lo) <= np.spacing(np.abs(k[..., 0])).astype(np.float64) / 2)


def test_bssn_constraint_convergence_order_unchanged(cuda):
    """|H| in 2 < r < 5 after a short evolution of Brill-Lindquist data
    (m = 0.5 at z = +-0.5) on Spherical grids at two resolutions: the
    convergence order is FD4's, and the same in compensated precision as in
    FP64 (the reference's |H| resolution-scaling check,
    Tutorial-Start_to_Finish-BSSNCurvilinear-Two_BHs_Collide.ipynb:1637-1673)."""
    import torch
    from nrpytutorial_gb300 import Evolution, Grid
    T = 0.2
    orders = {}
    for prec in ("fp64", "compensated"):
        norms = []
        for Nr, Nth in ((48, 24), (96, 48)):
            G = Grid("Spherical", (Nr, Nth, 4), FD_order=4, NGHOSTS=3, RMAX=8.0, eta=2.0)
            ev = Evolution("BSSN", G, precision=prec, device=cuda)
            ev.initial_data_brill_lindquist(0.5, (0, 0, 0.5), 0.5, (0, 0, -0.5))
            ev.apply_bcs(ev.y_n)
            ev.enforce_detgammabar(ev.y_n)
            dt0 = G.find_timestep(0.5)
            n = int(np.ceil(T / dt0))
            for _ in range(n):
                ev.step(T / n)
            H = ev.hamiltonian()[0].cpu().numpy()
            g = 3
            r = np.asarray(G.xx[0])[None, None, :] * np.ones_like(H)
            m = np.zeros_like(H, dtype=bool)
            m[g:-g, g:-g, g:-g] = True
            m &= (r > 2.0) & (r < 5.0)
            norms.append(float(np.sqrt(np.mean(H[m] ** 2))))
        orders[prec] = float(np.log2(norms[0] / norms[1]))
    print("convergence orders", orders)
    assert 3.0 < orders["fp64"] < 5.0, orders
    assert abs(orders["compensated"] - orders["fp64"]) < 0.05, orders
