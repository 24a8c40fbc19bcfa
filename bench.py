#!/usr/bin/env python
"""Benchmark: BSSN gridpoint-RHS/s of the RK4 method-of-lines step.

Workload (the reference's BSSN curvilinear configuration): SinhSpherical
reference metric (AMPL=64, SINHW=0.2), Nr x Ntheta x Nphi = 128 x 64 x 16
interior points + 3 ghost zones, 4th-order FD, RK4, Brill-Lindquist data
(m = 0.5, 0.5 at z = +-0.5), 1+log lapse, covariant Gamma-driver (eta = 2),
CFL 0.5.  One step = one RK4 step = 4 RHS evaluations per interior point
(the reference's gp/s definition, Nxx0*Nxx1*Nxx2*4 per step,
Tutorial-Start_to_Finish-BSSNCurvilinear-Two_BHs_Collide.ipynb:1165-1166).

  python bench.py [--gpus N --steps K --warmup W]      GB300 arm
  python bench.py --impl reference ...                 the reference's own
      generated C (OpenMP, host cores) on the same workload

`value` is the compensated mixed-precision step (FP32 RHS on FP32 (hi, lo)
stage pairs, FP64 RK state) with its error against the FP64 run stated in
the line; the FP64 run, the plain FP32-stage run and the other
configurations (Cartesian 256^3 FD6, 512 batched ScalarWave evolutions, the
Maxwell and ScalarWave adjoint gradients) are reported beside it.

Prints one JSON line (rank 0).  For N > 1 (torchrun) every rank evolves an
independent replica ("replicas only": one evolution does not shard here).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W = dict(name="BSSN SinhSpherical 128x64x16 FD4 RK4 Brill-Lindquist", coord="SinhSpherical",
         Nxx=(128, 64, 16), fd=4, ng=3, AMPL=64.0, SINHW=0.2, eta=2.0, CFL=0.5,
         m1=0.5, pos1=(0.0, 0.0, 0.5), m2=0.5, pos2=(0.0, 0.0, -0.5))
METRIC = "BSSN gridpoint-RHS/s (RK4 step), mixed precision at stated error vs FP64"
KO_STRENGTH = 0.1  # Kreiss-Oliger strength of the dissipated runs (BaikalETK's default_KO_strength)
UNIT = "gridpoint-RHS/s"
# Algorithmic bytes per interior point of the step's dominant kernel, the
# fused staged BSSN kernel of substep 1 (Ricci computed in the block, then
# the RHSs, k stored for the separate RK update kernel): stage input read
# and k written, 24 gfs as compensated FP32 pairs: 24 x 8 + 24 x 8 = 384 B.
DOM_BYTES_COMP = 24 * 8 + 24 * 8
# and of the step's RK update kernel (substep 1): k, y_n and running total
# read, running total and stage value written: 24 x 5 x 8 = 960 B.
UPDATE_BYTES_COMP = 24 * 5 * 8
# DRAM bytes (read + write) per launch of the two, L2 flushed before each
# launch as in the timing: one ncu capture of the launches inside the
# "roofline_rhs" and "roofline_update" ranges
# (profiles/bssn_split_step_compensated_roofline_traffic.md), means over the
# captured launches.
DOM_TRAFFIC_COMP = 45.13e6  # 42.90 MB read + 2.23 MB written
UPDATE_TRAFFIC_COMP = 81.75e6  # 79.13 MB read + 2.62 MB written
# Arithmetic of one BSSN Ricci + RHS evaluation at a SinhSpherical FD4 point,
# counted from the reference-generated C (+ - * / outside load lines,
# approximate): ~5.5k in rhs_eval and ~3.6k in Ricci_eval.  The FP32
# non-tensor nominal rate: 152 SMs x 128 lanes x 2 flops x 2.07 GHz.
BSSN_FLOPS_PER_POINT = 9100
FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12
RHS_BYTES_F64_FUSED = 24 * 8 + 6 * 8 + 24 * 8 + 24 * 16 + 24 * 8
RHS_BYTES_F64 = (24 + 6 + 24) * 8


def state_errors(a, b, c0, names):
    """Errors of state `a` against the FP64 state `b` (interior points,
    (ngf, ...) tensors; c0 the common initial state): whole-state normwise
    relative error, and per field the relative error, the error relative to
    the field's change since c0, and the max-norm relative error.  Fields
    whose FP64 norm is below 1e-6 of the largest field norm are identically
    zero in the continuum (symmetry) and are reported but not ranked."""
    import torch
    a = a.double()
    d = a - b
    norms = [float(torch.linalg.vector_norm(b[i])) for i in range(b.shape[0])]
    big = max(norms)
    fields = {}
    for i, n in enumerate(names):
        nd = float(torch.linalg.vector_norm(d[i]))
        nch = float(torch.linalg.vector_norm(b[i] - c0[i]))
        fields[n] = {"rel_l2": nd / max(norms[i], 1e-300), "rel_l2_of_change": nd / max(nch, 1e-300),
                     "rel_max": float(d[i].abs().max()) / max(float(b[i].abs().max()), 1e-300),
                     "norm_fp64": norms[i], "significant": norms[i] >= 1e-6 * big}
    sig = [f for f in fields.values() if f["significant"]]
    return {"state_rel_l2": float(torch.linalg.vector_norm(d)) / float(torch.linalg.vector_norm(b)),
            "max_rel_l2_significant_fields": max(f["rel_l2"] for f in sig),
            "max_rel_max_significant_fields": max(f["rel_max"] for f in sig),
            "max_rel_l2_of_change_significant_fields": max(f["rel_l2_of_change"] for f in sig),
            "fields": fields}


PROFILE_N3 = PROFILE_N4 = PROFILE_N5 = None  # --profile-sizes: smaller configurations 3-5


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.lines = []
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(self.index)],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        sm, smax, reasons, pw = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            c = [x.strip() for x in ln.split(",")]
            if len(c) < 9:
                continue
            try:
                sm.append(float(c[1]))
                smax.append(float(c[2]))
                pw.append(float(c[3]))
            except ValueError:
                continue
            for n, v in zip(names, c[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_median": float(np.median(pw)) if pw else None}


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


# --------------------------------------------------------------- GB300 arm
def run_gpu(args):
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    from nrpytutorial_gb300 import Evolution, Grid, _lib
    lib = _lib.load()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    G = Grid(W["coord"], W["Nxx"], FD_order=W["fd"], NGHOSTS=W["ng"], AMPL=W["AMPL"], SINHW=W["SINHW"],
             eta=W["eta"])
    nint = G.n_interior()
    dt = G.find_timestep(W["CFL"])
    ev = Evolution("BSSN", G, precision="fp64", device=dev)
    ev.initial_data_brill_lindquist(W["m1"], W["pos1"], W["m2"], W["pos2"])
    ev.apply_bcs(ev.y_n)
    ev.enforce_detgammabar(ev.y_n)
    y0 = ev.y_n.clone()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2
    K, Wm = args.steps, args.warmup
    sampler = ClockSampler(local)
    sampler.start()

    def timed_replays(replay, n):
        ev_s = [torch.cuda.Event(enable_timing=True) for _ in range(n)]
        ev_e = [torch.cuda.Event(enable_timing=True) for _ in range(n)]
        for k in range(n):
            flush.zero_()                    # evict L2 between timed steps (untimed)
            ev_s[k].record()
            replay()
            ev_e[k].record()
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in zip(ev_s, ev_e)) / 1e3

    def run(e, label=None):
        """K graph-replayed RK4 steps from y0 after Wm warm-up steps; returns
        (seconds, kernel launches per step).  With a label, one more warm-up
        replay runs inside an NVTX range of that name (for per-kernel
        profiles of one step; outside the timed region)."""
        e.y_n.copy_(y0)
        for _ in range(Wm):
            e.step(dt)
        e.y_n.copy_(y0)
        l0 = lib.nrgpu_kernel_launch_count()
        e.step(dt)
        lps = lib.nrgpu_kernel_launch_count() - l0
        replay = e.capture(dt, n_steps=1)
        for _ in range(Wm):
            replay()
        if label:
            torch.cuda.nvtx.range_push(label)
            replay()
            torch.cuda.nvtx.range_pop()
        e.y_n.copy_(y0)
        barrier()
        t = timed_replays(replay, K)
        barrier()
        if world > 1:
            import torch.distributed as dist
            tt = torch.tensor([t], device=dev)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            t = float(tt.item())
        return t, lps

    def kernel_time(fn, reps=20):
        ts = []
        for r in range(reps + 3):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            if r >= 3:
                ts.append(a.elapsed_time(b) / 1e3)
        return float(np.mean(ts))

    # ---- FP64 (parity mode)
    t64, lps64 = run(ev, "headline_step_fp64")
    y64 = ev.y_n.clone()
    H64 = ev.l2_norm(ev.hamiltonian(y64))
    g = W["ng"]
    c0 = y0[:, g:-g, g:-g, g:-g]

    # ---- headline: compensated mixed precision
    evc = Evolution("BSSN", G, precision="compensated", device=dev)
    tc, lps = run(evc, "headline_step_compensated")
    finite = bool(torch.isfinite(evc.y_n).all().item())
    comp_err = state_errors(evc.y_n[:, g:-g, g:-g, g:-g], y64[:, g:-g, g:-g, g:-g], c0, ev.gf_names)
    Hc = ev.l2_norm(ev.hamiltonian(evc.y_n))
    value = world * K * nint * 4 / tc
    launches = lps * K

    # ---- the FP64-accumulation form: FP32 RHS on pair stages, RK update and
    # det(gammabar) rescale in FP64 arithmetic
    evf = Evolution("BSSN", G, precision="compensated_fp64rk", device=dev)
    tf, lpsf = run(evf)
    f_err = state_errors(evf.y_n[:, g:-g, g:-g, g:-g], y64[:, g:-g, g:-g, g:-g], c0, ev.gf_names)
    Hf = ev.l2_norm(ev.hamiltonian(evf.y_n))

    # ---- error legs over the configuration's 200 steps (untimed), whatever K is
    def evolve_from_y0(e, n):
        e.y_n.copy_(y0)
        e.capture(dt, n_steps=n)()
        torch.cuda.synchronize()
        return e.y_n[:, g:-g, g:-g, g:-g].clone()

    N200 = 200
    y64_200 = evolve_from_y0(ev, N200)
    H64_200 = ev.l2_norm(ev.hamiltonian(ev.y_n))
    err200 = {}
    for name, e in (("compensated", evc), ("compensated_fp64rk", evf)):
        ye = evolve_from_y0(e, N200)
        er = state_errors(ye, y64_200, c0, ev.gf_names)
        err200[name] = {"state_rel_l2": er["state_rel_l2"],
                        "max_rel_l2_significant_fields": er["max_rel_l2_significant_fields"],
                        "max_rel_max_significant_fields": er["max_rel_max_significant_fields"],
                        "H_l2": ev.l2_norm(ev.hamiltonian(e.y_n)), "H_l2_fp64": H64_200}
    del evf

    # ---- plain FP32 stage buffers, for comparison
    evm = Evolution("BSSN", G, precision="mixed", device=dev)
    tm, _ = run(evm)
    mix_err = state_errors(evm.y_n[:, g:-g, g:-g, g:-g], y64[:, g:-g, g:-g, g:-g], c0, ev.gf_names)
    Hm = ev.l2_norm(ev.hamiltonian(evm.y_n))
    del evm

    # ---- Kreiss-Oliger dissipation switched on, FP64 and compensated
    Gk = Grid(W["coord"], W["Nxx"], FD_order=W["fd"], NGHOSTS=W["ng"], AMPL=W["AMPL"], SINHW=W["SINHW"],
              eta=W["eta"], diss_strength=KO_STRENGTH)
    ek = Evolution("BSSN", Gk, precision="fp64", device=dev)
    tk64, _ = run(ek)
    yk64 = ek.y_n.clone()
    ekc = Evolution("BSSN", Gk, precision="compensated", device=dev)
    tkc, _ = run(ekc)
    ko_err = state_errors(ekc.y_n[:, g:-g, g:-g, g:-g], yk64[:, g:-g, g:-g, g:-g], c0, ev.gf_names)
    ekc.y_n.copy_(y0)
    ekc.step(dt)
    t_rhs_kc = kernel_time(lambda: ekc.substep_rhs(dt, 1, 2))
    ko = {"diss_strength": KO_STRENGTH, "compensated_ms_per_step": tkc / K * 1e3,
          "fp64_ms_per_step": tk64 / K * 1e3, "speedup_vs_fp64": tk64 / tkc,
          "compensated_rhs_kernel_ms": t_rhs_kc * 1e3,
          "state_rel_l2": ko_err["state_rel_l2"],
          "max_rel_l2_significant_fields": ko_err["max_rel_l2_significant_fields"],
          "fp64_state_change_from_dissipation": float(torch.linalg.vector_norm(yk64 - y64)
                                                      / torch.linalg.vector_norm(y64 - y0))}
    del ek, ekc, yk64

    # ---- the step's kernels alone (substep 1, fused RK update, after a step)
    evc.y_n.copy_(y0)
    evc.step(dt)
    t_ric_c = kernel_time(lambda: evc.substep_rhs(dt, 1, 1))
    t_rhs_c = kernel_time(lambda: evc.substep_rhs(dt, 1, 2))
    # the launches the roofline's traffic capture selects: the step's fused
    # Ricci + RHS kernel storing k, and its RK update kernel
    torch.cuda.nvtx.range_push("roofline_rhs")
    t_step_c = kernel_time(lambda: evc.substep_rhs(dt, 1, 3))
    torch.cuda.nvtx.range_pop()
    torch.cuda.nvtx.range_push("roofline_update")
    t_upd_c = kernel_time(lambda: evc.substep_rhs(dt, 1, 4))
    torch.cuda.nvtx.range_pop()
    ev.y_n.copy_(y0)
    ev.step(dt)
    t_ric_64 = kernel_time(lambda: ev.substep_rhs(dt, 1, 1))
    t_rhs_64 = kernel_time(lambda: ev.substep_rhs(dt, 1, 2))

    # ---- psi4 extraction (FP64 diagnostic): whole grid, and one shell + its l <= 8 modes
    import ctypes as C
    p4 = torch.zeros((2,) + tuple(y64.shape[1:]), dtype=torch.float64, device=dev)
    modes = torch.zeros(2 * 77, dtype=torch.float64, device=dev)
    ish = W["ng"] + W["Nxx"][0] // 2

    def psi4_shell():
        ev.psi4(y64, (ish, ish + 1), out=p4)
        _lib.check(lib.BSSN_psi4_spinweightm2_decomposition(C.byref(G.params), _lib.ptr(p4), ish, 8,
                                                            _lib.ptr(modes)), "psi4 modes")

    t_p4 = kernel_time(lambda: ev.psi4(y64, out=p4))
    t_p4s = kernel_time(psi4_shell)
    psi4_info = {"full_grid_ms": t_p4 * 1e3, "points_per_s": nint / t_p4,
                 "shell_plus_modes_ms": t_p4s * 1e3, "shell_points": W["Nxx"][1] * W["Nxx"][2], "l_max": 8}

    # ---- end to end through the C ABI with host buffers (H2D + step + D2H per step)
    host = torch.empty(y0.shape, dtype=torch.float64, pin_memory=True)
    host.copy_(y0.cpu())
    hn = host.numpy()
    evc.evolve_host(hn, dt, 1)  # warm
    host.copy_(y0.cpu())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(K):
        evc.evolve_host(hn, dt, 1)
    te2e = time.perf_counter() - t0
    clocks = sampler.stop()

    hbm, src = peaks()
    achieved = nint * DOM_BYTES_COMP / t_step_c / 1e9
    achieved_upd = nint * UPDATE_BYTES_COMP / t_upd_c / 1e9
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": Wm,
        "ms_per_step": tc / K * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 RHS on compensated f32 (hi,lo) stage pairs; RK accumulation in float-float (48-bit "
                 "significand) on the FP32 pipe; f64 RK state between steps",
        "data": "synthetic: Brill-Lindquist initial data computed on the GPU",
        "config": {"workload": W["name"], "Nxx": list(W["Nxx"]), "NGHOSTS": W["ng"], "FD_order": W["fd"],
                   "interior_points": nint, "parallelism": "replicas" if world > 1 else "single",
                   "l2": "flushed (256 MB write) before every timed step",
                   "launch": "each step replays a CUDA graph of its %d kernel launches" % lps},
        "error_vs_fp64_200_steps": err200,
        "fp64_accumulation_form": {
            "what": "FP32 RHS on FP32 (hi, lo) pair stages; RK4 accumulation, y_n, running total and the "
                    "det(gammabar) rescale in FP64 arithmetic (NRGPU_PREC_COMPENSATED_FP64RK)",
            "value": world * K * nint * 4 / tf, "unit": UNIT, "ms_per_step": tf / K * 1e3,
            "launches_per_step": lpsf, "speedup_vs_fp64": t64 / tf,
            "error_vs_fp64": {"after_steps": K, "state_rel_l2": f_err["state_rel_l2"],
                              "max_rel_l2_significant_fields": f_err["max_rel_l2_significant_fields"],
                              "max_rel_max_significant_fields": f_err["max_rel_max_significant_fields"],
                              "H_l2": Hf}},
        "error_vs_fp64": {"after_steps": K, "state_rel_l2": comp_err["state_rel_l2"],
                          "max_rel_l2_significant_fields": comp_err["max_rel_l2_significant_fields"],
                          "max_rel_max_significant_fields": comp_err["max_rel_max_significant_fields"],
                          "H_l2_fp64": H64, "H_l2": Hc},
        "gpu_launches": int(launches),
        "state_finite": finite,
        "e2e": {"value": world * K * nint * 4 / te2e, "unit": UNIT,
                "h2d_bytes_per_step": int(y0.numel() * 8), "d2h_bytes_per_step": int(y0.numel() * 8),
                "path": "MoL_evolve_host (C ABI), compensated precision, pinned host FP64 state, 1 step per call "
                        "(repeated identical calls replay a CUDA graph of the two copies and the step)"},
        "roofline": {"bound": "hbm", "kernel": "bssn staged_kernel (FUSED variant: Ricci in the block, then the "
                                               "RHSs, k stored) of substep 1, compensated FP32 pairs",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_source": src, "traffic": DOM_TRAFFIC_COMP, "traffic_unit": "bytes per launch",
                     "bytes_per_point": DOM_BYTES_COMP,
                     "launch_ms": t_step_c * 1e3,
                     "note": "the step's dominant kernel (TMA-staged shared-memory finite differences, 8 warps "
                             "per SM) is issue/latency bound by the BSSN algebra, not by HBM; HBM fraction "
                             "reported as asked. The RK update runs in the separate kernel of roofline_update",
                     "issue": {"issue_slots_busy": 0.320, "fma_pipe_busy": 0.182, "warps_active_per_sm": 7.7,
                               "dram_throughput_of_peak": 0.041,
                               "source": "ncu --set full of the same kernel (substep 0), "
                                         "profiles/bssn_split_step_kernels_compensated_sinhsph_128x64x16.md",
                               "fp32_flops_per_point": BSSN_FLOPS_PER_POINT,
                               "achieved_fp32_tflops": nint * BSSN_FLOPS_PER_POINT / t_step_c / 1e12,
                               "fp32_nominal_tflops": FP32_NOMINAL_TFLOPS,
                               "frac_of_fp32_nominal": nint * BSSN_FLOPS_PER_POINT / t_step_c / 1e12
                                                       / FP32_NOMINAL_TFLOPS}},
        "roofline_update": {"bound": "hbm", "kernel": "rk4_update_interior_kernel<float2, 1> (float-float RK4 "
                                                      "update of substep 1 at the interior points)",
                            "achieved": achieved_upd, "peak": hbm, "unit": "GB/s", "frac": achieved_upd / hbm,
                            "peak_source": src, "traffic": UPDATE_TRAFFIC_COMP, "traffic_unit": "bytes per launch",
                            "bytes_per_point": UPDATE_BYTES_COMP, "launch_ms": t_upd_c * 1e3},
        "kernels_ms": {"compensated": {"ricci": t_ric_c * 1e3, "rhs": t_rhs_c * 1e3, "fused_ricci_rhs": t_step_c * 1e3,
                                       "rk_update": t_upd_c * 1e3},
                       "fp64": {"ricci": t_ric_64 * 1e3, "rhs": t_rhs_64 * 1e3}},
        "fp64": {"value": world * K * nint * 4 / t64, "unit": UNIT, "ms_per_step": t64 / K * 1e3,
                 "launches_per_step": lps64, "H_l2": H64,
                 "rhs_kernel_GBps": nint * RHS_BYTES_F64_FUSED / t_rhs_64 / 1e9,
                 "note": "FP64 BSSN is FP64-pipe bound on GB300 (FP32:FP64 = 64:1)"},
        "speedup_vs_fp64": t64 / tc,
        "mixed_fp32_stages": {"value": world * K * nint * 4 / tm, "ms_per_step": tm / K * 1e3,
                              "speedup_vs_fp64": t64 / tm, "state_rel_l2": mix_err["state_rel_l2"],
                              "max_rel_l2_significant_fields": mix_err["max_rel_l2_significant_fields"],
                              "H_l2": Hm},
        "kreiss_oliger": ko,
        "psi4": psi4_info,
        "compensated_fields": {k: {"rel_l2": v["rel_l2"], "rel_max": v["rel_max"]}
                               for k, v in comp_err["fields"].items() if v["significant"]},
        "clocks": clocks,
    }
    del evc
    torch.cuda.empty_cache()
    out["scalarwave_cartesian_64"] = run_config1(dev)
    torch.cuda.empty_cache()
    if args.config3_steps > 0:
        out["mixed_cartesian_256"] = run_config3(dev, args.config3_steps, flush, N=PROFILE_N3 or 256)
        torch.cuda.empty_cache()
    if args.config4_steps > 0:
        out["batched_scalarwave_512"] = run_config4(dev, args.config4_steps, flush, n=PROFILE_N4 or 512)
        torch.cuda.empty_cache()
    if not args.profile_sizes:
        out["convergence_order_H"] = convergence_orders(dev)
    if args.config5_steps > 0:
        a5 = run_config5(dev, args.config5_steps, N=PROFILE_N5 or 128)
        out["adjoint_maxwell_128"] = a5
        out["adjoint_over_forward"] = a5["adjoint_over_forward"]
    if args.sw_adjoint_steps > 0:
        out["adjoint_scalarwave_sinhsph"] = run_scalarwave_adjoint(dev, args.sw_adjoint_steps)
    if args.bl_gradient_steps > 0:
        out["gradient_bssn_brill_lindquist"] = run_bl_gradient(dev, args.bl_gradient_steps)
    if not args.profile_sizes and world == 1:
        out["slab_two_ranks_one_gpu"] = run_slab_local(dev)
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(args)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_config1(dev, N=64, nsteps=100):
    """Configuration 1: ScalarWave Cartesian [-10,10]^3, 64^3 + 2 ghosts, FD4,
    RK4, CFL 0.5, 100 steps, plane wave u = sin(k.x - |k|t), k = (2 pi/20)(1,1,1),
    quadratic-extrapolation outer BCs, FP64 (and compensated precision beside
    it); errors against the exact solution on the central half of the z
    midplane (Tutorial-Start_to_Finish-ScalarWave.ipynb:514-520) at t = 2.5
    (4th-order regime; the 32^3 run gives the order) and at the final
    t = 15.625, where the extrapolation boundary's growing mode has reached
    the centre (in the reference's own run too)."""
    import torch
    import oracle.grid as og
    import oracle.wave_maxwell as ow
    from nrpytutorial_gb300 import Evolution, Grid

    def central(e, n, g):
        m = n + 2 * g
        lo, hi = int(m * 0.25) + 1, int(np.ceil(m * 0.75))
        return float(np.abs(e[m // 2, lo:hi, lo:hi]).max())

    res = {"workload": "ScalarWave Cartesian %d^3 FD4 RK4 CFL 0.5 plane wave k=(2pi/20)(1,1,1), %d steps"
                       % (N, nsteps)}
    for prec in ("fp64", "compensated"):
        errs = {}
        for n in (N // 2, N):
            G = Grid("Cartesian", (n, n, n), FD_order=4, NGHOSTS=2)
            gp = og.GridParams("Cartesian", (n, n, n), 2, 4)
            ev = Evolution("ScalarWave", G, precision=prec, device=dev)
            y0 = torch.tensor(ow.plane_wave(gp, 0.0), device=dev)
            dt = 0.5 * gp.dxx[0]
            steps = nsteps * n // N
            n25 = int(round(2.5 / dt))
            ev.y_n.copy_(y0)
            ev.capture(dt, n_steps=n25)()
            e25 = central(ev.y_n[0].cpu().numpy() - ow.plane_wave(gp, n25 * dt)[0], n, 2)
            rep = ev.capture(dt, n_steps=1)
            ev.y_n.copy_(y0)
            for _ in range(3):
                rep()
            ev.y_n.copy_(y0)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(steps):
                rep()
            b.record()
            torch.cuda.synchronize()
            t = a.elapsed_time(b) / 1e3
            ef = central(ev.y_n[0].cpu().numpy() - ow.plane_wave(gp, steps * dt)[0], n, 2)
            errs[n] = {"err_t2.5": e25, "err_final": ef, "steps": steps, "seconds": t,
                       "gp_per_s": n ** 3 * 4 * steps / t, "ms_per_step": t / steps * 1e3}
            del ev
        r = dict(errs[N])
        r["convergence_order_t2.5"] = float(np.log2(errs[N // 2]["err_t2.5"] / errs[N]["err_t2.5"]))
        r["coarse_%d" % (N // 2)] = errs[N // 2]
        res[prec] = r
    res["note"] = ("steps are CUDA-graph replays of one RK4 step (launch-bound at this size); L2 not flushed "
                   "(the 2.5 MB state stays in L2, as it does in a running evolution)")
    return res


def run_config3(dev, K, flush, N=256):
    """Configuration 3: BSSN Cartesian [-10,10]^3, 256^3 interior, FD6 (4 ghosts),
    RK4, Brill-Lindquist with masses ~U[0.3,0.7] at z = +-U[0.3,1.0] (seeded);
    FP32 storage and RHS with FP64 RK accumulation, det(gammabar) rescale and
    constraint norms, compared field by field against the FP64 run."""
    import torch
    from nrpytutorial_gb300 import Evolution, Grid
    rng = np.random.default_rng(3)
    m1, m2 = rng.uniform(0.3, 0.7, 2)
    z1, z2 = rng.uniform(0.3, 1.0), -rng.uniform(0.3, 1.0)
    G = Grid("Cartesian", (N, N, N), FD_order=6, NGHOSTS=4, domain=(-10.0, 10.0), eta=2.0)
    nint = G.n_interior()
    dt = G.find_timestep(0.5)
    e64 = Evolution("BSSN", G, precision="fp64", device=dev)
    e64.initial_data_brill_lindquist(m1, (0, 0, z1), m2, (0, 0, z2))
    e64.apply_bcs(e64.y_n)
    e64.enforce_detgammabar(e64.y_n)
    y0 = e64.y_n.clone()
    res = {"workload": "BSSN Cartesian %d^3 FD6 RK4 Brill-Lindquist m=(%.4f,%.4f) z=(%.4f,%.4f), seed 3"
                       % (N, m1, m2, z1, z2), "steps": K, "dt": dt}
    times, errs, H = {}, {}, {}
    g = 4
    B = e64.y_n[:, g:-g, g:-g, g:-g]
    C0 = y0[:, g:-g, g:-g, g:-g]
    for prec in ("fp64", "mixed", "compensated"):
        e = e64 if prec == "fp64" else Evolution("BSSN", G, precision=prec, device=dev)
        e.y_n.copy_(y0)
        e.step(dt)  # warm-up
        e.y_n.copy_(y0)
        torch.cuda.synchronize()
        tt = 0.0
        for _ in range(K):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            e.step(dt)
            b.record()
            torch.cuda.synchronize()
            tt += a.elapsed_time(b) / 1e3
        times[prec] = tt
        H[prec] = e64.l2_norm(e64.hamiltonian(e.y_n))
        if prec != "fp64":
            errs[prec] = state_errors(e.y_n[:, g:-g, g:-g, g:-g], B, C0, e64.gf_names)
            if prec == "mixed":
                emix = e
            else:
                del e
                torch.cuda.empty_cache()
    res["fp64_gp_per_s"] = K * nint * 4 / times["fp64"]
    res["ms_per_step_fp64"] = times["fp64"] / K * 1e3
    res["H_l2_fp64"] = H["fp64"]
    for prec in ("mixed", "compensated"):
        r = {"gp_per_s": K * nint * 4 / times[prec], "ms_per_step": times[prec] / K * 1e3,
             "speedup_vs_fp64": times["fp64"] / times[prec], "H_l2": H[prec]}
        r.update(errs[prec])
        res[prec] = r
    # FP32 rhs kernel alone at this size: algorithmic bytes 54 x 4 B per point
    y32 = emix.y_n.float()
    aux = torch.zeros((6,) + G.shape, dtype=torch.float32, device=dev)
    rhs = torch.zeros_like(y32)
    emix.ricci_eval(y32, aux)
    ts = []
    for r in range(8):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        emix.rhs_eval_given_ricci(y32, aux, rhs)
        b.record()
        torch.cuda.synchronize()
        if r >= 3:
            ts.append(a.elapsed_time(b) / 1e3)
    t = float(np.mean(ts))
    hbm, _ = peaks()
    res["rhs_f32_kernel"] = {"launch_ms": t * 1e3, "bytes_per_point": 54 * 4,
                             "achieved_GBps": nint * 216 / t / 1e9, "frac_of_hbm": nint * 216 / t / 1e9 / hbm}
    del e64, emix
    return res


def run_config4(dev, K, flush, n=512):
    """Configuration 4: 512 independent ScalarWave evolutions on Spherical
    grids (RMAX 10), Nr ~ U{32..160} (seeded), Ntheta 32, Nphi 8, FD4, RK4 with
    each instance's own CFL-0.5 time step, Gaussian pulses
    u = A exp(-(r-r0)^2/w^2) with A ~ U[0.1,1], r0 ~ U[1,4], w ~ U[0.5,2].
    FP32 RHS / FP64 accumulation (plain FP32 stages and compensated FP32
    pairs), K steps replayed from one CUDA graph, tile autotuned; compared
    with the FP64 batch over the same K steps."""
    import torch
    from nrpytutorial_gb300 import _lib
    from nrpytutorial_gb300.batch import ScalarWaveBatch
    rng = np.random.default_rng(4)
    Nr = rng.integers(32, 161, n)
    A, r0, w = rng.uniform(0.1, 1.0, n), rng.uniform(1.0, 4.0, n), rng.uniform(0.5, 2.0, n)
    res = {"workload": "%d x ScalarWave Spherical Nr~U{32..160} x 32 x 8 FD4 RK4, seed 4" % n, "steps": K}
    runs = {}
    lib = _lib.load()
    for prec in ("fp64", "mixed", "compensated"):
        B = ScalarWaveBatch(Nr, 32, 8, CoordSystem="Spherical", RMAX=10.0, precision=prec, device=dev)
        B.initial_data_gaussian(A, r0, w)
        tile = B.autotune(reps=3)
        y0 = B.y_n.clone()
        replay = B.capture(n_steps=K)
        c0 = lib.nrgpu_kernel_launch_count()
        B.step()
        launches = lib.nrgpu_kernel_launch_count() - c0
        B.y_n.copy_(y0)
        flush.zero_()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        replay()
        b.record()
        torch.cuda.synchronize()
        t = a.elapsed_time(b) / 1e3
        runs[prec] = (B, t)
        res[prec] = {"tile": {"tx": tile[0], "ty": tile[1], "grid": tile[2], "rhs_launch_ms": tile[3]},
                     "seconds": t, "ms_per_step": t / K * 1e3, "launches_per_step": int(launches)}
        del replay
    B64, t64 = runs["fp64"]
    nint = B64.interior_points()
    hbm, _ = peaks()
    # algorithmic bytes per interior point of one RK4 step (2 gfs; stage input,
    # y_n, running total, stage output per substep, plus the pair split):
    bpp = {"fp64": 2 * (24 + 40 + 40 + 32), "mixed": 2 * (20 + 32 + 32 + 28), "compensated": 2 * (32 + 40 + 40 + 32 + 16)}
    for prec in ("fp64", "mixed", "compensated"):
        t = runs[prec][1]
        res[prec].update({"gp_updates_per_s": K * nint / t, "instance_steps_per_s": K * n / t,
                          "bytes_per_point_step": bpp[prec], "achieved_GBps": K * nint * bpp[prec] / t / 1e9,
                          "frac_of_hbm": K * nint * bpp[prec] / t / 1e9 / hbm})
        if prec != "fp64":
            Bp = runs[prec][0]
            errs = [float(torch.linalg.vector_norm(Bp.instance(i)[0] - B64.instance(i)[0]) /
                          torch.linalg.vector_norm(B64.instance(i)[0])) for i in range(n)]
            res[prec].update({"speedup_vs_fp64": t64 / t, "u_rel_l2_vs_fp64_max_over_instances": max(errs),
                              "u_rel_l2_vs_fp64_median": float(np.median(errs))})
    res.update({"interior_points": nint, "total_points_per_gf_set": B64.total})
    del runs, B64
    torch.cuda.empty_cache()
    return res


def convergence_orders(dev):
    """|H| in 2 < r < 5 after t = 0.2 of Brill-Lindquist data (m = 0.5 at
    z = +-0.5) on Spherical grids 48x24x4 and 96x48x4 (RMAX 8, FD4): the
    convergence order log2(|H|_coarse / |H|_fine), FP64 and both mixed forms."""
    from nrpytutorial_gb300 import Evolution, Grid
    T, out = 0.2, {}
    for prec in ("fp64", "compensated", "compensated_fp64rk"):
        norms = []
        for Nr, Nth in ((48, 24), (96, 48)):
            G = Grid("Spherical", (Nr, Nth, 4), FD_order=4, NGHOSTS=3, RMAX=8.0, eta=2.0)
            ev = Evolution("BSSN", G, precision=prec, device=dev)
            ev.initial_data_brill_lindquist(0.5, (0, 0, 0.5), 0.5, (0, 0, -0.5))
            ev.apply_bcs(ev.y_n)
            ev.enforce_detgammabar(ev.y_n)
            n = int(np.ceil(T / G.find_timestep(0.5)))
            for _ in range(n):
                ev.step(T / n)
            H = ev.hamiltonian()[0].cpu().numpy()
            r = np.asarray(G.xx[0])[None, None, :] * np.ones_like(H)
            m = np.zeros_like(H, dtype=bool)
            m[3:-3, 3:-3, 3:-3] = True
            m &= (r > 2.0) & (r < 5.0)
            norms.append(float(np.sqrt(np.mean(H[m] ** 2))))
        out[prec] = {"H_rms_coarse": norms[0], "H_rms_fine": norms[1], "order": float(np.log2(norms[0] / norms[1]))}
    return out


def run_config5(dev, K, N=128):
    """Configuration 5: Maxwell System I, Cartesian [-10,10]^3 at 128^3, FD4,
    FP64, K RK4 steps (CFL 0.5) from toroidal-dipole data with seeded
    amplitude and width parameters; observable = L2 norm of E over the
    sphere r = 8 (32 x 64 points) and the evolution; gradient with respect
    to (amp, lam) by the discrete adjoint, checkpoints every 20 steps,
    checked against central differences with h = 1e-6."""
    import torch
    from nrpytutorial_gb300 import Grid
    from nrpytutorial_gb300.adjoint import ExtractionSphere, MaxwellExtraction
    rng = np.random.default_rng(5)
    amp, lam = rng.uniform(0.5, 1.5), rng.uniform(0.5, 1.5)
    G = Grid("Cartesian", (N, N, N), FD_order=4, NGHOSTS=3, domain=(-10.0, 10.0))
    m = MaxwellExtraction(G, ExtractionSphere(8.0, 32, 64), n_steps=K, checkpoint_every=20, device=dev)
    m.forward(amp, lam)  # warm-up
    m.gradient()

    def timed(f):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        r = f()
        b.record()
        torch.cuda.synchronize()
        return r, a.elapsed_time(b) / 1e3

    J, t_fwd = timed(lambda: m.forward(amp, lam))
    g, t_bwd = timed(m.gradient)
    h = 1e-6
    fd = [(m.forward(amp + h, lam) - m.forward(amp - h, lam)) / (2 * h),
          (m.forward(amp, lam + h) - m.forward(amp, lam - h)) / (2 * h)]
    rel = [abs(g[i] - fd[i]) / abs(fd[i]) for i in range(2)]
    nint = N ** 3
    return {"workload": "Maxwell System I Cartesian [-10,10]^3 %d^3 FD4 FP64, %d RK4 steps, toroidal dipole "
                        "amp=%.6f lam=%.6f (seed 5), |E| on sphere r=8 (32x64), checkpoints every 20" % (N, K, amp, lam),
            "J": J, "grad": [float(v) for v in g], "grad_central_fd_h1e-6": [float(v) for v in fd],
            "grad_rel_err_vs_fd": rel, "forward_s": t_fwd, "adjoint_s": t_bwd,
            "adjoint_over_forward": t_bwd / t_fwd, "gradient_over_forward": (t_fwd + t_bwd) / t_fwd,
            "forward_gp_updates_per_s": K * nint / t_fwd, "checkpoints": len(m.checkpoints)}



def run_scalarwave_adjoint(dev, K, Nxx=(128, 32, 64)):
    """ScalarWave on a SinhSpherical grid (AMPL 10, SINHW 0.2, FD4, FP64),
    K RK4 steps (CFL 0.5) from a Gaussian pulse u = A exp(-(r-r0)^2/w^2)
    with seeded (A, r0, w); observable = L2 norm of u over the radial shell
    at two thirds of the radial extent and the evolution; gradient with
    respect to (A, r0, w) by the discrete adjoint (checkpoints every 20
    steps), checked against central differences with h = 1e-6.  The pulse
    sits 1.2 widths inside the shell (r0 = r_shell - 1.2 w)."""
    import torch
    from nrpytutorial_gb300 import Grid
    from nrpytutorial_gb300.adjoint import ScalarWaveExtraction
    import ctypes as C
    from nrpytutorial_gb300 import _lib
    G = Grid("SinhSpherical", Nxx, FD_order=4, NGHOSTS=3, AMPL=10.0, SINHW=0.2)
    i0 = 3 + (2 * Nxx[0]) // 3
    x = (C.c_double * 3)()
    _lib.check(_lib.load().xx_to_Cart(C.byref(G.params), None, i0, 3, 3, x), "xx_to_Cart")
    r_shell = float(np.sqrt(x[0] ** 2 + x[1] ** 2 + x[2] ** 2))
    # the pulse centred 1.2 widths inside the shell, so that no component of
    # the gradient vanishes (a shell at the pulse centre has dJ/dw ~ 0)
    rng = np.random.default_rng(7)
    A, w = rng.uniform(0.5, 1.5), rng.uniform(0.3, 0.6)
    r0 = r_shell - 1.2 * w
    m = ScalarWaveExtraction(G, i0, n_steps=K, checkpoint_every=20, device=dev)
    m.forward(A, r0, w)  # warm-up
    m.gradient()

    def timed(f):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        r = f()
        b.record()
        torch.cuda.synchronize()
        return r, a.elapsed_time(b) / 1e3

    J, t_fwd = timed(lambda: m.forward(A, r0, w))
    g, t_bwd = timed(m.gradient)
    h = 1e-6
    fd = []
    for k in range(3):
        p, q = [A, r0, w], [A, r0, w]
        p[k] += h
        q[k] -= h
        fd.append((m.forward(*p) - m.forward(*q)) / (2 * h))
    rel = [abs(g[i] - fd[i]) / abs(fd[i]) for i in range(3)]
    nint = Nxx[0] * Nxx[1] * Nxx[2]
    return {"workload": "ScalarWave SinhSpherical AMPL=10 SINHW=0.2 %dx%dx%d FD4 FP64, %d RK4 steps, Gaussian "
                        "A=%.6f r0=%.6f w=%.6f (seed 7; r0 = r_shell - 1.2 w), u on the shell i0=%d (r=%.6f), "
                        "checkpoints every 20" % (Nxx + (K, A, r0, w, i0, r_shell)),
            "J": J, "grad": [float(v) for v in g], "grad_central_fd_h1e-6": [float(v) for v in fd],
            "grad_rel_err_vs_fd": rel, "forward_s": t_fwd, "adjoint_s": t_bwd,
            "adjoint_over_forward": t_bwd / t_fwd, "gradient_over_forward": (t_fwd + t_bwd) / t_fwd,
            "forward_gp_updates_per_s": K * nint / t_fwd, "checkpoints": len(m.checkpoints)}



def run_bl_gradient(dev, K, Nxx=(64, 32, 8)):
    """Brill-Lindquist parameter gradient by forward mode: BSSN SinhSpherical
    (AMPL 64, SINHW 0.2, FD4, FP64), K RK4 steps (CFL 0.5) from BL data
    m1 = 0.5 at z = 0.5, m2 = 0.3 at z = -0.7; observable = L2 norm of
    alpha - 1 over the radial shell at two thirds of the radial extent and the
    evolution; gradient with respect to (m1, m2, z1, z2) in one
    tangent-linear pass (4 tangents), checked against central differences
    (h = 1e-6) of the same discrete evolution."""
    import torch
    from nrpytutorial_gb300 import Grid
    from nrpytutorial_gb300.tangent import BrillLindquistGradient
    G = Grid("SinhSpherical", Nxx, FD_order=4, NGHOSTS=3, AMPL=64.0, SINHW=0.2, eta=2.0)
    i0 = 3 + (2 * Nxx[0]) // 3
    m = BrillLindquistGradient(G, i0, n_steps=K, params=("m1", "m2", "z1", "z2"), device=dev)
    # unequal masses off the symmetric configuration, so that no component of
    # the gradient vanishes by symmetry
    base = (0.5, (0.0, 0.0, 0.5), 0.3, (0.0, 0.0, -0.7))
    m.value_only(*base)  # warm-up

    def timed(f):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        r = f()
        b.record()
        torch.cuda.synchronize()
        return r, a.elapsed_time(b) / 1e3

    J0, t_fwd = timed(lambda: m.value_only(*base))
    (J, g), t_tan = timed(lambda: m.value_and_gradient(*base))
    theta = np.array([base[0], base[2], *base[1], *base[3]], dtype=float)
    h = 1e-6
    fd = []
    for q in (0, 1, 4, 7):
        tp, tm = theta.copy(), theta.copy()
        tp[q] += h
        tm[q] -= h
        fd.append((m.value_only(*BrillLindquistGradient.unpack(tp)) -
                   m.value_only(*BrillLindquistGradient.unpack(tm))) / (2 * h))
    rel = [abs(g[k] - fd[k]) / max(abs(fd[k]), 1e-300) for k in range(4)]
    return {"workload": "BSSN SinhSpherical AMPL=64 SINHW=0.2 %dx%dx%d FD4 FP64, %d RK4 steps, Brill-Lindquist "
                        "m1=0.5 at z=0.5, m2=0.3 at z=-0.7, alpha-1 on the shell i0=%d" % (Nxx + (K, i0)),
            "method": "forward mode: state + 4 tangents (d/dm1, d/dm2, d/dz1, d/dz2) in one pass",
            "J": J, "J_plain": J0, "grad": [float(v) for v in g], "grad_central_fd_h1e-6": [float(v) for v in fd],
            "grad_rel_err_vs_fd": rel, "forward_s": t_fwd, "tangent_pass_s": t_tan,
            "gradient_over_forward": t_tan / t_fwd}



def run_slab_local(dev, K=5):
    """The slab decomposition's own cost on one GPU: the headline grid's FP64
    BSSN step split into two i2 slabs driven in this process (LocalComm:
    per substep both ranks' kernels, the cross-rank parity gathers and the
    halo exchange, all on this GPU), against the one-grid step; bit-for-bit
    agreement checked.  On two GPUs the ranks' kernels would run
    concurrently; here they run one after the other, so the difference of the
    two times is the exchange overhead."""
    import torch
    from nrpytutorial_gb300 import Evolution, Grid
    from nrpytutorial_gb300.slab import LocalComm, SlabEvolution
    G = Grid(W["coord"], W["Nxx"], FD_order=W["fd"], NGHOSTS=W["ng"], AMPL=W["AMPL"], SINHW=W["SINHW"],
             eta=W["eta"])
    ev = Evolution("BSSN", G, precision="fp64", device=dev)
    ev.initial_data_brill_lindquist(W["m1"], W["pos1"], W["m2"], W["pos2"])
    ev.apply_bcs(ev.y_n)
    ev.enforce_detgammabar(ev.y_n)
    sl = SlabEvolution("BSSN", G, LocalComm(2), device=dev)
    sl.set_state(ev.y_n)
    dt = G.find_timestep(0.5)
    ev.step(dt)
    sl.step(dt)  # warm-up

    def timed(f):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(K):
            f()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / K

    t1 = timed(lambda: ev.step(dt))
    t2 = timed(lambda: sl.step(dt))
    parts = sorted(sl.owned_state(r) for r in range(2))
    same = bool(torch.equal(torch.cat([p for _, p in parts], dim=1), ev.y_n))
    # the same steps replayed from CUDA graphs: launch and host costs out
    g1 = ev.capture(dt, 1)
    g2 = sl.capture(dt, 1)
    t1g = timed(g1)
    t2g = timed(g2)
    return {"workload": "BSSN headline grid FP64, split into 2 slabs of 8 i2 planes on one GPU (LocalComm)",
            "one_grid_ms_per_step": t1, "two_slabs_ms_per_step": t2, "exchange_overhead_ms": t2 - t1,
            "graph_one_grid_ms_per_step": t1g, "graph_two_slabs_ms_per_step": t2g,
            "graph_exchange_overhead_ms": t2g - t1g, "bit_identical_to_one_grid": same}


# ------------------------------------------------------------ CPU reference
class RefStepper:
    """The reference's generated Ricci_eval/rhs_eval/enforce (OpenMP -Ofast
    build) plus our C restatement of its RK update and BCs."""

    def __init__(self, flavour="fast"):
        import ctypes as C
        import oracle.bcs as ob
        import oracle.grid as og
        from oracle import ref_build
        from oracle.ref import RefKernels, available
        ref_build.build_if_present()
        self.gp = gp = og.GridParams(W["coord"], W["Nxx"], W["ng"], W["fd"], AMPL=W["AMPL"], SINHW=W["SINHW"],
                                     eta=W["eta"])
        cfg = "bssn_sinhsph_fd4"
        if not available(cfg, flavour):
            raise FileNotFoundError("reference-generated kernels for %s not built" % cfg)
        self.kind = "reference"
        extra = {"BH1_mass": W["m1"], "BH1_posn_x": W["pos1"][0], "BH1_posn_y": W["pos1"][1],
                 "BH1_posn_z": W["pos1"][2], "BH2_mass": W["m2"], "BH2_posn_x": W["pos2"][0],
                 "BH2_posn_y": W["pos2"][1], "BH2_posn_z": W["pos2"][2]}
        self.R = RefKernels(cfg, gp, flavour, extra=extra)
        self.mol = C.CDLL(ref_build.MOL_LIB)
        layers = ob.build_bcstruct(gp)
        ob_start, od, os_, ib_start, idd, isrc, ipar = [0], [], [], [0], [], [], []
        for outer, (d, s, p) in layers:
            for arr in outer:
                od += list(arr[:, 0]); os_ += list(arr[:, 1])
            ob_start.append(len(od))
            idd += list(d); isrc += list(s)
            ipar += [int(sum((1 << t) for t in range(10) if row[t] < 0)) for row in p]
            ib_start.append(len(idd))
        i32 = lambda v: np.ascontiguousarray(np.array(v, dtype=np.int32))
        self.bc = [i32(ob_start), i32(od), i32(os_), i32(ib_start), i32(idd), i32(isrc), i32(ipar)]
        from nrpytutorial_gb300.grid import SYSTEM_GFS
        self.par = np.array(SYSTEM_GFS["BSSN"][1], dtype=np.int8)
        self.ntot = int(np.prod(gp.shape))
        shape = (24,) + gp.shape
        self.y = self.R.initial_data(shape)
        self.post(self.y)
        self.rt = np.zeros(shape)
        self.k = [np.zeros(shape), np.zeros(shape)]
        self.aux = np.zeros((6,) + gp.shape)
        self.dt = og.find_timestep(gp, W["CFL"])

    def post(self, g):
        import ctypes as C
        ptrs = [a.ctypes.data_as(C.POINTER(C.c_int)) for a in self.bc]
        self.mol.ref_apply_bcs(C.c_int(self.gp.NGHOSTS), ptrs[0], ptrs[1], ptrs[2], ptrs[3], ptrs[4], ptrs[5],
                               ptrs[6], C.c_int(24), self.par.ctypes.data_as(C.POINTER(C.c_int8)),
                               C.c_longlong(self.ntot), g.ctypes.data_as(C.POINTER(C.c_double)))
        self.R.lib.ref_enforce_detgammabar_constraint(*self.R._x(), g.ctypes.data_as(C.POINTER(C.c_double)))

    def step(self):
        import ctypes as C
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        n = C.c_longlong(24 * self.ntot)
        ins = [self.y, self.k[0], self.k[1], self.k[0]]
        outs = [self.k[0], self.k[1], self.k[0], self.k[1]]
        for s in range(4):
            self.R.lib.ref_Ricci_eval(*self.R._x(), dp(ins[s]), dp(self.aux))
            self.R.lib.ref_rhs_eval(*self.R._x(), dp(self.aux), dp(ins[s]), dp(outs[s]))
            self.mol.ref_rk4_update(C.c_int(s), C.c_double(self.dt), n, dp(self.y), dp(self.rt), dp(outs[s]))
            self.post(self.y if s == 3 else outs[s])


class ShipStepper:
    """The reference's BSSN step in the form its Brill-Lindquist driver ships
    (Tutorial-Start_to_Finish-BSSNCurvilinear-Two_BHs_Collide.ipynb):
    rfm_precompute, SIMD-macro loops (scalar where the host has no AVX/SSE2),
    finite_difference_functions.h, the generated RK_MoL.h with Ricci_eval,
    rhs_eval, apply_bcs_curvilinear and enforce_detgammabar_constraint, and
    the reference's own bcstruct set-up -- generated by oracle/gen_ref_ship.py,
    compiled with the reference's -Ofast -fopenmp -funroll-loops -march=native."""

    NAME = "bssn_ship_sinhsph_fd4"

    def __init__(self, flavour="fast"):
        import ctypes as C
        import oracle.grid as og
        from oracle import ref_build
        ref_build.build_if_present()
        path = os.path.join(ref_build.LIB, "%s.%s.so" % (self.NAME, flavour))
        if not os.path.exists(path):
            raise FileNotFoundError("shipping-form reference step not built (%s)" % path)
        self.lib = lib = C.CDLL(path)
        lib.ship_setup.argtypes = [C.c_int] * 3 + [C.c_double] * 7
        lib.ship_step.argtypes = [C.c_double]
        lib.ship_ntot.restype = C.c_longlong
        lib.ship_setup(*W["Nxx"], W["AMPL"], W["SINHW"], W["eta"], W["m1"], W["pos1"][2], W["m2"], W["pos2"][2])
        gp = og.GridParams(W["coord"], W["Nxx"], W["ng"], W["fd"], AMPL=W["AMPL"], SINHW=W["SINHW"], eta=W["eta"])
        self.dt = og.find_timestep(gp, W["CFL"])
        self.kind = "reference"
        self.form = ("shipping form: rfm_precompute, SIMD-macro loops, FD functions, generated RK_MoL.h + "
                     "apply_bcs_curvilinear + enforce_detgammabar_constraint")

    def step(self):
        self.lib.ship_step(self.dt)


def ref_stepper():
    """The reference's step in its shipping form, else the no-precompute form."""
    try:
        return ShipStepper()
    except Exception:  # noqa: BLE001
        st = RefStepper()
        st.form = "no-precompute form: Read_xxs rhs_eval/Ricci_eval + C restatement of RK update and BCs"
        return st


def time_stepper(st, budget_s, max_steps=1000):
    """Steps of a CPU stepper for about budget_s seconds after one warm-up step."""
    st.step()
    n, t0 = 0, time.perf_counter()
    while n < max_steps and time.perf_counter() - t0 < budget_s:
        st.step()
        n += 1
    return n, time.perf_counter() - t0


def cpu_baseline(args, budget_s=10.0):
    """The reference's own C on the host cores, a bounded (~10 s) sample;
    the no-precompute form is timed beside it."""
    nint = int(np.prod(W["Nxx"]))
    try:
        st = ref_stepper()
        n, dt = time_stepper(st, budget_s)
        out = {"value": n * nint * 4 / dt, "unit": UNIT, "cores": os.cpu_count(), "kind": "reference",
               "sample": "%d full RK4 steps of the workload (%.1f s), reference-generated C in its %s; "
                         "gcc -Ofast -fopenmp, OMP threads=%s" %
                         (n, dt, st.form, os.environ.get("OMP_NUM_THREADS", "all"))}
        if isinstance(st, ShipStepper):
            try:
                n2, dt2 = time_stepper(RefStepper(), budget_s / 2)
                out["no_precompute_form"] = {"value": n2 * nint * 4 / dt2, "steps": n2, "seconds": dt2}
            except Exception as e:  # noqa: BLE001
                out["no_precompute_form"] = {"unavailable": str(e)[:200]}
        return out
    except Exception as e:  # noqa: BLE001
        return port_baseline(str(e))


def port_baseline(why):
    """numpy oracle on one z-slab of the workload (bounded sample)."""
    import oracle.bssn as obs
    import oracle.grid as og
    gp = og.GridParams(W["coord"], (W["Nxx"][0], W["Nxx"][1], 2), W["ng"], W["fd"], AMPL=W["AMPL"],
                       SINHW=W["SINHW"], eta=W["eta"])
    rng = np.random.default_rng(0)
    f = 0.01 * rng.random((24,) + gp.shape)
    f[obs.GF["cf"]] += 1
    f[obs.GF["alpha"]] += 1
    t0 = time.perf_counter()
    obs.rhs_grid(gp, f)
    dt = time.perf_counter() - t0
    n = W["Nxx"][0] * W["Nxx"][1] * 2
    return {"value": n / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "numpy oracle, one RHS evaluation on a 2-plane slab (%s)" % why[:120]}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    nint = int(np.prod(W["Nxx"]))
    try:
        st = ref_stepper()
    except Exception as e:  # noqa: BLE001
        print(json.dumps({"impl": "reference", "unavailable": "reference-generated kernels not built: %s" % e}))
        return
    for _ in range(max(0, args.warmup)):
        st.step()
    times = []
    t_start = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        st.step()
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > args.ref_budget_s:
            break
    k = len(times)
    tt = sum(times)
    value = k * nint * 4 / tt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": k,
        "warmup": args.warmup, "ms_per_step": tt / k * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic: Brill-Lindquist (reference-generated initial_data)",
        "config": {"workload": W["name"], "Nxx": list(W["Nxx"]), "NGHOSTS": W["ng"], "FD_order": W["fd"]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "reference",
                         "sample": "%d of %d requested full RK4 steps (time budget %.0f s), reference-generated "
                                   "C in its %s (gcc -Ofast -fopenmp -funroll-loops -march=native)"
                                   % (k, args.steps, args.ref_budget_s, st.form)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--ref-budget-s", type=float, default=90.0)
    ap.add_argument("--config3-steps", type=int, default=4,
                    help="RK4 steps of the 256^3 Cartesian mixed-vs-FP64 comparison (0 skips it)")
    ap.add_argument("--profile-sizes", action="store_true",
                    help="small configurations 3-5 (96^3, 64 instances, 48^3) for profiler captures")
    ap.add_argument("--config5-steps", type=int, default=300,
                    help="RK4 steps of the Maxwell 128^3 adjoint-gradient run (0 skips it)")
    ap.add_argument("--bl-gradient-steps", type=int, default=40,
                    help="RK4 steps of the Brill-Lindquist forward-mode gradient run (0 skips it)")
    ap.add_argument("--sw-adjoint-steps", type=int, default=1000,
                    help="RK4 steps of the SinhSpherical ScalarWave adjoint-gradient run (0 skips it)")
    ap.add_argument("--config4-steps", type=int, default=400,
                    help="RK4 steps of the 512-instance batched ScalarWave run (0 skips it)")
    args = ap.parse_args()
    global PROFILE_N3, PROFILE_N4, PROFILE_N5
    if args.profile_sizes:
        PROFILE_N3, PROFILE_N4, PROFILE_N5 = 96, 64, 48
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
