"""Benchmark of the Chorin projection time step on one GB300 (replicas on N GPUs).

Workload (the DFG channel at h = 0.005): synthetic channel mesh with a cylinder, ~84k triangles,
N = 169,672 P2 velocity nodes, P = 42,741 P1 pressure nodes; inflow peak 6.0 (U_max = 1.5),
nu = 1e-3, tau = 1e-4 (the reference's default time step; the 5e-4 of the DFG config lies outside the
explicit scheme's stability region at this resolution: tau <= 2 / (nu * lambda_max(M^-1 K)) = 1.98e-4),
pressure solved to 1e-8 relative residual with CG preconditioned by multicolor
symmetric Gauss-Seidel.  A "step" is one full time step (FastConvection + diffusion operator, SpMM,
tentative mass solve, divergence, pressure solve, gradient, final mass solve, Dirichlet updates).

``value`` is steps/s of the mixed-precision stepper (FP32 SpMV/sweeps/inner CG, FP64 refinement,
dots and state) with everything resident in HBM; ``e2e`` is the same through the C ABI with the
state uploaded from and downloaded to host memory every step.  The FP64 stepper is reported in
``variants``.  ``--impl reference`` times the CPU restatement of the path (the C oracle, FP64).
"""

from __future__ import annotations

import argparse
import gzip
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

H = 0.005
PEAK = 6.0        # reference inflow peakVelocity = 4 * U_max with U_max = 1.5
NU = 1e-3
TAU = 1e-4        # stable: explicit diffusion limit at h = 0.005 is 1.98e-4
PRES_TOL = 1e-8
VEL_TOL = 1e-8
METRIC = "channel-flow steps/s: mixed-prec vs FP64 CG on 1 GB300 at 1e-8 rel; SpMV/CG HBM GB/s"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


PRESSURE_GUESSES = {0: "previous solution", 1: "2 p(n-1) - p(n-2)",
                    2: "projection onto <= {} earlier solutions, Kp_int-orthonormal (Fischer 1998)"}
MASS_SOLVES = {1: "PCG, multicolor SGS", 2: "PCG, Jacobi", 3: "Chebyshev, Jacobi (a priori iteration count)",
               4: "Chebyshev, Jacobi, from the previous step's solution (a priori count from the initial residual)"}


def make_mesh(tmpdir: str, h: float, seed: int = 0) -> str:
    from nsfemoptim_gb300 import meshgen
    path = os.path.join(tmpdir, f"channel_h{h}_s{seed}.msh")
    meshgen.write_gmsh41(path, meshgen.dfg_channel(h, seed=seed))
    return path


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu: int):
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(gpu), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx = max(mx, float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def run_cpu_reference(mesh_path: str, steps: int, warmup: int, vel_method: int = 1, pres_guess: int = 0,
                      pres_basis: int = 0, snapshot_step: int = 0):
    """Time the oracle's FP64 Chorin step (the CPU restatement of the reference path) on every host
    thread (its OpenMP build; the single-thread build if that cannot be compiled): `warmup` steps
    from rest, then `steps` timed ones.  The thread count is left in CPU_THREADS.  Returns steps/s,
    the timed seconds, the context and (u, p, forces) after `snapshot_step` steps in all (taken
    outside the timing; the final state if 0)."""
    global CPU_THREADS
    import oracle
    oracle.build()
    m = oracle.Mesh(mesh_path)
    ctx = oracle.Context(m, PEAK, True)
    ch = oracle.Chorin(ctx, NU, TAU, vel_method=vel_method, vel_max_iters=500, vel_tol=VEL_TOL, pres_max_iters=5000,
                       pres_tol=PRES_TOL, mt=True, pres_guess=pres_guess, pres_basis=pres_basis)
    CPU_THREADS = ch.threads
    snap = None

    def take():
        u, p = ch.state()
        return u, p, oracle.forces(m, u, p, NU)

    for k in range(warmup):
        ch.step()
        if k + 1 == snapshot_step:
            snap = take()
    dt = 0.0
    for k in range(steps):
        t0 = time.perf_counter()
        ch.step()
        dt += time.perf_counter() - t0
        if warmup + k + 1 == snapshot_step:
            snap = take()
    return steps / dt, dt, ctx, snap if snap is not None else take()


CPU_THREADS = 1                    # host threads of the last CPU-oracle timing
ACC_STEPS = 100                    # accuracy run: mixed vs FP64 from rest
ACC_CHECKPOINTS = (4, 25, 50, 100)  # steps at which the fields are compared


def accuracy_run(G, ctx, mesh, stepper, torch, stream):
    """Mixed-precision and FP64 steppers from rest for ACC_STEPS steps: relative L2 field
    differences at the checkpoints, the drag/lift time series (both on the device, FP64) and the
    pressure-solve iterations of every step."""
    sp = stream.cuda_stream
    runs = {}
    iters = {}
    for name, prec in (("fp64", G.NSF_PREC_F64), ("mixed", G.NSF_PREC_MIXED)):
        st = stepper(prec)
        fn = G.Forces(mesh, st)
        F = torch.zeros((ACC_STEPS, 2), dtype=torch.float64, device="cuda")
        states = {}
        its = []
        with torch.cuda.stream(stream):
            for k in range(ACC_STEPS):
                st.step(1, sp)
                fn.into(F[k], sp)
                its.append(int(st.stats()["pres_iters"]))
                if k + 1 in ACC_CHECKPOINTS:
                    states[k + 1] = st.state()
        torch.cuda.synchronize()
        runs[name] = (F.cpu().numpy(), states)
        iters[name] = its
        del fn, st

    def rel(a, b):
        import numpy as np
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    import numpy as np
    F64, S64 = runs["fp64"]
    FMX, SMX = runs["mixed"]
    # coefficients c = 2 F / (U_mean^2 D) with U_mean = 2/3 U_max = PEAK / 6, D = 0.1
    cscale = 2.0 / ((PEAK / 6.0) ** 2 * 0.1)
    out = {
        "steps": ACC_STEPS,
        "field_rel_l2_mixed_vs_fp64": {str(k): {"u": rel(SMX[k][0], S64[k][0]), "p": rel(SMX[k][1], S64[k][1])}
                                       for k in ACC_CHECKPOINTS},
        "drag_max_rel_err_mixed_vs_fp64": float(np.abs(FMX[:, 0] - F64[:, 0]).max() / np.abs(F64[:, 0]).max()),
        "lift_max_err_mixed_vs_fp64_rel_to_max_drag": float(np.abs(FMX[:, 1] - F64[:, 1]).max() /
                                                            np.abs(F64[:, 0]).max()),
        "c_drag_fp64_last": float(cscale * F64[-1, 0]),
        "c_lift_fp64_last": float(cscale * F64[-1, 1]),
        "pressure_iterations": {k: {"mean": round(float(np.mean(v)), 1), "max": int(np.max(v)),
                                    "mean_last_50": round(float(np.mean(v[-50:])), 1), "last_10": v[-10:]}
                                for k, v in iters.items()},
    }
    return out, (S64[4][0], S64[4][1], F64[3])


def bench_small(args):
    """The small plain-FP64 configuration: synthetic channel at h = 0.02 (the reference does not
    ship that mesh; the generator makes it), U_max = 0.3 (peak 1.2), nu = 1e-3, tau = 1e-3, 2000
    steps from rest, pressure PCG-SGS to 1e-10 relative.  GPU FP64 and mixed steppers over all
    steps; the CPU oracle (FP64, one thread) on a bounded sample of the same run from rest."""
    import numpy as np
    import torch

    import nsfemoptim_gb300 as G
    import oracle

    h, peak, nu, tau, steps = 0.02, 1.2, 1e-3, 1e-3, args.small_steps
    tmp = tempfile.mkdtemp()
    try:
        path = make_mesh(tmp, h, 0)
        mesh = G.load_gmsh(path)
        ctx = G.build_chorin_context(mesh, peak)
        stream = torch.cuda.Stream()
        sp = stream.cuda_stream
        res = {}
        for name, prec in (("fp64", G.NSF_PREC_F64), ("mixed", G.NSF_PREC_MIXED)):
            st = G.ChorinStepper(ctx, nu, tau, precision=prec, vel_method=1, vel_max_iters=500, vel_tol=1e-10,
                                 pres_max_iters=5000, pres_tol=1e-10, check_interval=8, use_graph=True,
                                 max_outer=4, inner_tol=1e-5)
            with torch.cuda.stream(stream):
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                st.step(steps, sp)
                e1.record(stream)
                torch.cuda.synchronize()
            t = e0.elapsed_time(e1) / 1e3
            u, p = st.state()
            res[name] = {"steps_per_s": round(steps / t, 2), "ms_per_step": round(1e3 * t / steps, 4),
                         "stats": st.stats(), "u": u, "p": p}
            del st
        # CPU oracle from rest on a bounded sample; its state is compared with a GPU FP64 run of
        # the same number of steps
        k = max(1, args.small_cpu_steps)
        oracle.build()
        om = oracle.Mesh(path)
        oc = oracle.Context(om, peak, True)
        ch = oracle.Chorin(oc, nu, tau, vel_method=1, vel_max_iters=500, vel_tol=1e-10, pres_max_iters=5000,
                           pres_tol=1e-10, mt=True)
        cpu_threads = ch.threads
        t0 = time.perf_counter()
        for _ in range(k):
            ch.step()
        cpu_t = time.perf_counter() - t0
        uo, po = ch.state()
        st = G.ChorinStepper(ctx, nu, tau, precision=G.NSF_PREC_F64, vel_method=1, vel_max_iters=500, vel_tol=1e-10,
                             pres_max_iters=5000, pres_tol=1e-10, use_graph=True)
        st.step(k)
        ug, pg = st.state()
    finally:
        shutil.rmtree(tmp, ignore_errors=True)

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    return {
        "metric": "config 1: plain FP64 Chorin projection, h=0.02 channel, steps/s (GPU FP64 drop-in)",
        "value": res["fp64"]["steps_per_s"], "unit": "steps/s", "n_gpus": 1, "steps": steps,
        "higher_is_better": True, "dtype": "f64", "data": "synthetic (seeded DFG channel mesh, h=0.02)",
        "config": {"workload": "DFG channel h=0.02, Umax=0.3, nu=1e-3, tau=1e-3, P2/P1, pressure PCG-SGS to 1e-10 rel",
                   "triangles": mesh.num_tri, "N": ctx.N, "P": ctx.P},
        "variants": {n: {kk: v for kk, v in r.items() if kk not in ("u", "p")} for n, r in res.items()},
        "mixed_vs_fp64_after_all_steps": {"u_rel_l2": rel(res["mixed"]["u"], res["fp64"]["u"]),
                                          "p_rel_l2": rel(res["mixed"]["p"], res["fp64"]["p"])},
        "cpu_baseline": {"value": round(k / cpu_t, 3), "unit": "steps/s", "cores": cpu_threads, "kind": "port",
                         "sample": f"the first {k} steps from rest, FP64 C oracle on {cpu_threads} host threads"},
        "fp64_vs_oracle": {"steps": k, "u_rel_l2": rel(ug, uo), "p_rel_l2": rel(pg, po)},
    }


ADJ_H, ADJ_PEAK, ADJ_NU, ADJ_TAU, ADJ_TOL = 0.01, 4.0, 1e-3, 5e-4, 1e-13
ADJ_METRIC = "adjoint drag gradient time (d/dnu + 16 inflow coefficients), h=0.01, 1000 steps"


def _adjoint_oracle_sample(path, k, theta, basis, g0, scale):
    """The FP64 CPU adjoint (C oracle, on every host thread) on the first k steps from rest, every
    step weighted scale / k.  Returns (seconds, J, dJ/dnu, dJ/dtheta); the thread count is left in
    CPU_THREADS."""
    global CPU_THREADS
    import numpy as np
    import oracle
    oracle.build()
    om = oracle.Mesh(path)
    oc = oracle.Context(om, ADJ_PEAK, True)
    w = np.full(k, scale / k)
    CPU_THREADS = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)) if oracle.lib_mt() else 1
    t0 = time.perf_counter()
    J, gnu, gdir, _ = oracle.adjoint_run(oc, om, ADJ_NU, ADJ_TAU, k, w, dir_vx=g0 + basis @ theta, vel_tol=ADJ_TOL,
                                         pres_tol=ADJ_TOL, solve_tol=ADJ_TOL, mt=True)
    return time.perf_counter() - t0, J, gnu, basis.T @ gdir


def bench_adjoint(args):
    """Config 5, the discrete-adjoint gradient.  Synthetic DFG channel at h = 0.01, U_max = 1.0
    (context peak 4.0), nu = 1e-3, tau = 5e-4, 1000 steps from rest; J = mean drag coefficient over
    the last 500 steps; parameters nu and 16 sine-series coefficients of the inflow perturbation,
    theta ~ N(0, 0.01^2) (seed 0).  Forward and adjoint CG solves to 1e-13 relative residual, FP64.
    A "step" of this line is one whole gradient evaluation (forward run with checkpoints every 50
    steps, then the reverse sweep with segment recomputation).  Checked against FP64 central
    differences (eps = 1e-6) of the GPU forward run and against the FP64 CPU adjoint (C oracle) on
    a bounded sample at the same mesh."""
    import numpy as np
    import torch

    import nsfemoptim_gb300 as G
    from nsfemoptim_gb300 import gradcheck as GC

    n = args.adjoint_steps
    tmp = tempfile.mkdtemp()
    try:
        path = make_mesh(tmp, ADJ_H, 0)
        mesh = G.load_gmsh(path)
        ctx = G.build_chorin_context(mesh, ADJ_PEAK)
        w = np.zeros(n)
        w[n // 2:] = 1.0 / (n - n // 2)
        precs = {"f64": G.NSF_PREC_F64, "mixedsolve": G.NSF_PREC_F64_MIXEDSOLVE}
        prec = precs[args.adjoint_precision]
        prob = GC.DragProblem(mesh, ctx, ADJ_PEAK, ADJ_NU, ADJ_TAU, n, w, n_coef=16, tol=ADJ_TOL,
                              checkpoint_interval=args.adjoint_checkpoint, precision=prec,
                              vel_method=args.adjoint_vel_method)
        theta = 0.01 * np.random.default_rng(0).standard_normal(16)
        launches0 = G.kernel_launches()
        for _ in range(max(0, args.adjoint_warmup)):
            prob.gradient(ADJ_NU, theta)
        clk = Clocks(0)
        t_grad, t_e2e, t_fwd, t_rev = [], [], [], []
        launches0 = G.kernel_launches()
        for _ in range(max(1, args.adjoint_reps)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            J, gnu, gth, gdir = prob.gradient(ADJ_NU, theta)
            t_e2e.append(time.perf_counter() - t0)
            s = prob.adjoint.stats()
            t_fwd.append(s["forward_ms"] / 1e3)
            t_rev.append(s["reverse_ms"] / 1e3)
            t_grad.append(t_fwd[-1] + t_rev[-1])
        launches = G.kernel_launches() - launches0
        clocks = clk.stop()
        reps = max(1, args.adjoint_reps)
        st = prob.adjoint.stats()
        variants = {}
        if args.adjoint_variants:
            other = [p for p in precs if p != args.adjoint_precision][0]
            for name, ck, pr, sn in (("keep_all_states", 0, prec, 0),
                                     (f"binomial_{args.adjoint_snapshots}_states", 0, prec, args.adjoint_snapshots),
                                     (f"precision_{other}", args.adjoint_checkpoint, precs[other], 0)):
                var = GC.DragProblem(mesh, ctx, ADJ_PEAK, ADJ_NU, ADJ_TAU, n, w, n_coef=16, tol=ADJ_TOL,
                                     checkpoint_interval=ck, precision=pr, vel_method=args.adjoint_vel_method,
                                     snapshots=sn)
                Jk, gnuk, gthk, _ = var.gradient(ADJ_NU, theta)
                sk = var.adjoint.stats()
                variants[name] = {
                    "gradient_s": round((sk["forward_ms"] + sk["reverse_ms"]) / 1e3, 3),
                    "forward_s": round(sk["forward_ms"] / 1e3, 3), "reverse_s": round(sk["reverse_ms"] / 1e3, 3),
                    "state_bytes": int(sk["state_bytes"]), "checkpoint_interval": ck, "snapshots": sn,
                    "recomputed_steps": int(sk["recomputed_steps"]),
                    "adjoint_pressure_cg_iters": int(sk["pres_iters"]), "adjoint_mass_cg_iters": int(sk["mass_iters"]),
                    "max_rel_diff_vs_headline": float(max(abs(gnuk - gnu) / abs(gnu),
                                                          np.abs(gthk - gth).max() / np.abs(gth).max()))}
                del var
        # central differences of the GPU forward run
        eps = 1e-6
        fd = {}
        if args.adjoint_fd:
            fnu = (prob.value(ADJ_NU + eps, theta) - prob.value(ADJ_NU - eps, theta)) / (2 * eps)
            fd["nu"] = {"adjoint": gnu, "fd": fnu, "rel_err": abs(fnu - gnu) / abs(gnu)}
            for k in args.adjoint_fd_coefs:
                e = np.zeros(16)
                e[k - 1] = eps
                fk = (prob.value(ADJ_NU, theta + e) - prob.value(ADJ_NU, theta - e)) / (2 * eps)
                fd[f"theta_{k}"] = {"adjoint": float(gth[k - 1]), "fd": fk,
                                    "rel_err": abs(fk - gth[k - 1]) / abs(gth[k - 1])}
        # the FP64 CPU adjoint on a bounded sample (first k steps, all weighted) vs the GPU adjoint
        k = args.adjoint_cpu_steps
        if k > 0:
            cpu_t, Jo, gnuo, gtho = _adjoint_oracle_sample(path, k, theta, prob.basis, prob.g0, prob.scale)
            small = GC.DragProblem(mesh, ctx, ADJ_PEAK, ADJ_NU, ADJ_TAU, k, np.full(k, 1.0 / k), n_coef=16,
                                   tol=ADJ_TOL, checkpoint_interval=0, precision=prec,
                                   vel_method=args.adjoint_vel_method)
            Js, gnus, gths, _ = small.gradient(ADJ_NU, theta)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    N, P = ctx.N, ctx.P
    h2d = 8 * (2 * N + P) + 8 * N + 16 * n
    d2h = 8 * N + 8 * N + 16 * N + 24 + 24
    grad_s = statistics.median(t_grad)
    line = {
        "metric": ADJ_METRIC, "value": round(grad_s, 3), "unit": "s", "n_gpus": 1, "steps": reps,
        "warmup": max(0, args.adjoint_warmup), "ms_per_step": round(1e3 * grad_s, 1), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded DFG channel mesh, h=0.01; inflow coefficients seeded N(0, 0.01^2))",
        "config": {"workload": f"adjoint drag gradient: DFG channel h={ADJ_H}, Umax=1.0, nu={ADJ_NU}, tau={ADJ_TAU}, "
                               f"{n} steps from rest, J = mean c_D over the last {n - n // 2} steps, "
                               f"grad wrt nu + 16 inflow sine coefficients",
                   "N": N, "P": P, "checkpoint_interval": args.adjoint_checkpoint, "solve_tol": ADJ_TOL,
                   "mass_solve": MASS_SOLVES[args.adjoint_vel_method],
                   "precision": {"f64": "FP64 operators and solves",
                                 "mixedsolve": "FP64 operators and state; FP32 CG inside FP64 residual replacement / "
                                               "refinement to the same FP64 tolerance"}[args.adjoint_precision],
                   "l2": "no flush: one step is a whole gradient (seconds), its working set re-read thousands of times"},
        "e2e": {"value": round(statistics.median(t_e2e), 3), "unit": "s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "breakdown": {"forward_s": round(statistics.median(t_fwd), 3), "reverse_s": round(statistics.median(t_rev), 3),
                      "recomputed_steps": int(st["recomputed_steps"]), "reverse_steps": int(st["reverse_steps"]),
                      "adjoint_mass_cg_iters": int(st["mass_iters"]), "adjoint_pressure_cg_iters": int(st["pres_iters"]),
                      "state_bytes": int(st["state_bytes"]), "forward_ms_per_step": round(statistics.median(t_fwd) * 1e3 / n, 3)},
        "gradient": {"J": J, "dJ_dnu": gnu, "dJ_dtheta": [float(x) for x in gth]},
        "fd_check_eps_1e-6": fd,
        "variants": variants,
    }
    if k > 0:
        line["cpu_baseline"] = {"value": round(cpu_t * n / k, 1), "unit": "s", "cores": CPU_THREADS, "kind": "port",
                                "sample": f"FP64 C oracle forward + adjoint over the first {k} steps from rest on "
                                          f"{CPU_THREADS} host threads, scaled by {n}/{k} to the {n}-step gradient "
                                          f"(the oracle keeps every state)"}
        line["gpu_vs_cpu_adjoint_sample"] = {"steps": k, "J_rel": abs(Js - Jo) / abs(Jo),
                                             "dnu_rel": abs(gnus - gnuo) / abs(gnuo),
                                             "dtheta_rel_l2": float(np.linalg.norm(gths - gtho) / np.linalg.norm(gtho))}
    if clocks:
        line["clocks"] = clocks
    return line


def bench_batch(args):
    """Batched instances: B independent channel flows on one h = 0.01 mesh, U_max ~ U[0.2, 1.5]
    (peak = 4 U_max) and nu ~ logU[5e-4, 2e-3] from seed 0, tau = 2e-4 (the explicit scheme's
    limit at h = 0.01 is 2 / (nu lambda_max(M^-1 K)) = 4e-4 for nu = 2e-3, so the configured 5e-4
    would diverge), mixed precision.  Each instance is a graph-captured stepper on its own stream
    whose solves stay inside thread-block clusters, so the instances run side by side; all steps
    of all instances are enqueued before anything waits.  The timed region (CUDA events: a start
    event every stream waits for, a stop event that waits for every stream) covers K steps of
    every instance.  Reported: aggregate instance-steps/s, against one instance alone."""
    import math

    import numpy as np
    import torch

    import nsfemoptim_gb300 as G

    B, K, W = args.batch, args.batch_steps, 3
    h, tau = 0.01, 2e-4
    rng = np.random.default_rng(0)
    umax = rng.uniform(0.2, 1.5, B)
    nus = np.exp(rng.uniform(math.log(5e-4), math.log(2e-3), B))
    tmp = tempfile.mkdtemp()
    old = os.environ.get("NSF_PCG_PATH")
    os.environ["NSF_PCG_PATH"] = "auto-cluster"
    try:
        path = make_mesh(tmp, h, 0)
        mesh = G.load_gmsh(path)
        # ---- batched: one context (peak 4.0 = 4 x U_max 1), each instance's inflow the context's
        # scaled by its U_max; every operation of the step one launch for all instances (nsf_batch)
        bctx = G.build_chorin_context(mesh, 4.0)
        bdir = np.stack([bctx.dir_vx * float(umax[b]) for b in range(B)])
        batch = G.Batch(bctx, nus, tau, dir_vx=bdir, vel_max_iters=500, vel_tol=VEL_TOL, pres_max_iters=5000,
                        pres_tol=PRES_TOL, use_graph=True, max_outer=4, inner_tol=1e-5,
                        pressure_guess=args.pressure_guess, pressure_basis=args.pressure_basis)
        bstream = torch.cuda.Stream()
        batch.step(W, bstream.cuda_stream)
        torch.cuda.synchronize()

        def tbatch(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(bstream)
            batch.launch(steps, bstream.cuda_stream)
            e1.record(bstream)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / 1e3

        k0 = G.kernel_launches()
        t_batch = tbatch(K)  # steps W+1 .. W+K: the window of the per-stream steppers
        batch_launches = G.kernel_launches() - k0
        batch.step(1, bstream.cuda_stream)
        t_batch2 = tbatch(K)  # steps W+K+2 .. W+2K+1: the window of the one-graph pack
        batch.step(1, bstream.cuda_stream)
        bstats = [batch.stats(b) for b in range(B)]
        del batch
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        # the FP64 drop-in on the same mesh (one instance, the reference's pressure guess)
        f64 = G.ChorinStepper(bctx, float(np.median(nus)), tau, precision=G.NSF_PREC_F64, vel_method=args.vel_method,
                              vel_max_iters=500, vel_tol=VEL_TOL, pres_max_iters=5000, pres_tol=PRES_TOL,
                              check_interval=8, use_graph=True, pressure_guess=0)
        f64.step(W, bstream.cuda_stream)
        torch.cuda.synchronize()
        e0.record(bstream)
        f64.launch(K, bstream.cuda_stream)
        e1.record(bstream)
        torch.cuda.synchronize()
        t_f64 = e0.elapsed_time(e1) / 1e3
        del f64
        t0 = time.perf_counter()
        steppers = []
        for b in range(B):
            ctx = G.build_chorin_context(mesh, 4.0 * float(umax[b]))
            steppers.append(G.ChorinStepper(ctx, float(nus[b]), tau, precision=G.NSF_PREC_MIXED, vel_method=args.vel_method,
                                            vel_max_iters=500, vel_tol=VEL_TOL, pres_max_iters=5000,
                                            pres_tol=PRES_TOL, check_interval=8, use_graph=True, max_outer=4,
                                            inner_tol=1e-5, pressure_guess=args.pressure_guess,
                                            pressure_basis=args.pressure_basis))
        setup_s = time.perf_counter() - t0
        streams = [torch.cuda.Stream() for _ in range(B)]
        for st, s in zip(steppers, streams):
            st.step(W, s.cuda_stream)  # captures each graph; warm-up
        torch.cuda.synchronize()
        master = torch.cuda.Stream()

        def run(group, steps):
            start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            start.record(master)
            ends = []
            for st, s in group:
                s.wait_event(start)
            for _ in range(steps):
                for st, s in group:
                    st.launch(1, s.cuda_stream)
            for st, s in group:
                e = torch.cuda.Event()
                e.record(s)
                master.wait_event(e)
                ends.append(e)
            stop.record(master)
            torch.cuda.synchronize()
            return start.elapsed_time(stop) / 1e3

        t_one = run([(steppers[0], streams[0])], K)
        t_all = run(list(zip(steppers, streams)), K)
        # the same instances as one pack: every instance's step a branch of one graph
        pack = G.Pack(steppers)
        pack.step(1, master.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(master)
        pack.step(K, master.cuda_stream)
        e1.record(master)
        torch.cuda.synchronize()
        t_pack = e0.elapsed_time(e1) / 1e3
        del pack
        # one synchronous step per instance: statistics and status
        status, pres_iters = [], []
        for st, s in zip(steppers, streams):
            st.step(1, s.cuda_stream)
            sd = st.stats()
            status.append(int(sd["status"]))
            pres_iters.append(int(sd["pres_iters"]))
    finally:
        if old is None:
            os.environ.pop("NSF_PCG_PATH", None)
        else:
            os.environ["NSF_PCG_PATH"] = old
        shutil.rmtree(tmp, ignore_errors=True)
    agg = B * K / t_all
    one = K / t_one
    agg_batch = B * K / t_batch
    f64_one = K / t_f64
    return {
        "metric": "config 4: batched channel instances (h=0.01), aggregate instance-steps/s",
        "value": round(agg_batch, 2), "unit": "instance-steps/s", "n_gpus": 1, "steps": K, "warmup": W,
        "batched": {"instance_steps_per_s": round(agg_batch, 2), "ms_per_step": round(1e3 * t_batch / K, 3),
                    "window": f"steps {W + 1}..{W + K} from rest (the per-stream steppers' window)",
                    "instance_steps_per_s_later_window": round(B * K / t_batch2, 2),
                    "later_window": f"steps {W + K + 2}..{W + 2 * K + 1} (the one-graph pack's window)",
                    "kernel_launches_per_step": round(batch_launches / K, 1),
                    "execution": "nsf_batch: one context, every operation of the step one launch for all "
                                 "instances (operator kernels instance-fastest, pressure solves one launch of "
                                 f"{B} clusters), graph-captured; the pressure guess of the other variants",
                    "pres_iters_range": [int(min(x["pres_iters"] for x in bstats)),
                                         int(max(x["pres_iters"] for x in bstats))],
                    "status_all_ok": all(int(x["status"]) == 0 for x in bstats)},
        "fp64_drop_in_one_instance_steps_per_s": round(f64_one, 2),
        "batched_mixed_over_fp64_drop_in": round(agg_batch / f64_one, 2),
        "higher_is_better": True, "dtype": "f32-inner/f64-refine",
        "data": "synthetic (seeded DFG channel mesh h=0.01; U_max, nu per instance from seed 0)",
        "config": {"workload": f"{B} instances, h=0.01, U_max~U[0.2,1.5], nu~logU[5e-4,2e-3], tau=2e-4, "
                               "pressure to 1e-8 rel", "instances": B, "setup_s": round(setup_s, 1),
                   "mass_solve": MASS_SOLVES[args.vel_method],
                   "pressure_guess": PRESSURE_GUESSES[args.pressure_guess].format(args.pressure_basis or 250),
                   "execution": "nsf_batch (batched kernels); per-stream steppers and the one-graph pack beside it"},
        "per_stream_steppers": {"instance_steps_per_s": round(agg, 2),
                                "execution": "one graph-captured stepper per instance on its own stream, "
                                             "cluster-resident solves"},
        "one_instance_steps_per_s": round(one, 2),
        "batched_over_one_instance": round(agg_batch / one, 2),
        "one_graph_pack": {"instance_steps_per_s": round(B * K / t_pack, 2),
                           "window": f"steps {W + K + 2}..{W + 2 * K + 1} from rest",
                           "execution": "all instances' steps as branches of one CUDA graph (nsf_pack), one launch "
                                        "per step"},
        "status_all_ok": all(s == 0 for s in status),
        "pres_iters_range": [min(pres_iters), max(pres_iters)],
    }


def bench_pack(args):
    """Uneven pack: 16 instances on each of three channel meshes (h = 0.025, 0.01, 0.005; synthetic,
    seed 0), U_max ~ U[0.2, 1.5] and nu ~ logU[5e-4, 2e-3] per instance (seed 1), mixed precision,
    mass solves of --vel-method, pressure to 1e-8, tau = 5e-5 (inside the explicit limit
    2 / (nu lambda_max(M^-1 K)) = 9.9e-5 of the finest mesh at nu = 2e-3).  All 48 time steps are
    branches of one CUDA graph (nsf_pack): one launch advances every instance, and every solve stays
    inside a thread-block cluster so the branches run side by side.  Timed: K launches (CUDA events
    on the launching stream).  Compared with the same 48 steppers stepped one after another."""
    import math

    import numpy as np
    import torch

    import nsfemoptim_gb300 as G

    per, K, W, tau = args.pack_per_mesh, args.pack_steps, 3, 5e-5
    hs = (0.025, 0.01, 0.005)
    rng = np.random.default_rng(1)
    tmp = tempfile.mkdtemp()
    old = os.environ.get("NSF_PCG_PATH")
    os.environ["NSF_PCG_PATH"] = "auto-cluster"
    try:
        t0 = time.perf_counter()
        steppers, meshes, sizes, draws = [], [], {}, []
        for h in hs:
            mesh = G.load_gmsh(make_mesh(tmp, h, 0))
            meshes.append(mesh)
            for _ in range(per):
                umax = float(rng.uniform(0.2, 1.5))
                nu = float(math.exp(rng.uniform(math.log(5e-4), math.log(2e-3))))
                draws.append((umax, nu))
                ctx = G.build_chorin_context(mesh, 4.0 * umax)
                sizes[h] = (ctx.N, ctx.P)
                steppers.append(G.ChorinStepper(ctx, nu, tau, precision=G.NSF_PREC_MIXED, vel_method=args.vel_method,
                                                vel_max_iters=500, vel_tol=VEL_TOL, pres_max_iters=5000,
                                                pres_tol=PRES_TOL, check_interval=8, use_graph=True, max_outer=4,
                                                inner_tol=1e-5, pressure_guess=args.pressure_guess,
                                                pressure_basis=args.pressure_basis))
        setup_s = time.perf_counter() - t0
        stream = torch.cuda.Stream()
        pack = G.Pack(steppers)
        pack.step(W, stream.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        pack.step(K, stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        t_pack = e0.elapsed_time(e1) / 1e3
        # the same steppers one after another (each its own graph), and one of each mesh alone
        e0.record(stream)
        for _ in range(K):
            for st in steppers:
                st.launch(1, stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        t_seq = e0.elapsed_time(e1) / 1e3
        alone = {}
        for i, h in enumerate(hs):
            st = steppers[i * per]
            e0.record(stream)
            st.launch(K, stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize()
            alone[str(h)] = round(K / (e0.elapsed_time(e1) / 1e3), 2)
        status = []
        for st in steppers:
            st.step(1, stream.cuda_stream)
            status.append(int(st.stats()["status"]))
        launches = G.kernel_launches()
        pack_kernels = pack.kernels_per_step()
        del pack
        # the same instances as three batches (one per mesh, nsf_batch) in one pack graph: every
        # operation one launch per mesh; the same step window as the pack of steppers
        batches = []
        for i, mesh in enumerate(meshes):
            um = np.array([d[0] for d in draws[i * per:(i + 1) * per]])
            nus = np.array([d[1] for d in draws[i * per:(i + 1) * per]])
            bctx = G.build_chorin_context(mesh, 4.0)
            batches.append(G.Batch(bctx, nus, tau, dir_vx=np.stack([bctx.dir_vx * u for u in um]), vel_max_iters=500,
                                   vel_tol=VEL_TOL, pres_max_iters=5000, pres_tol=PRES_TOL, use_graph=True,
                                   max_outer=4, inner_tol=1e-5, pressure_guess=args.pressure_guess,
                                   pressure_basis=args.pressure_basis))
        bpack = G.Pack(batches)
        bpack.step(W, stream.cuda_stream)
        torch.cuda.synchronize()
        e0.record(stream)
        bpack.step(K, stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        t_bpack = e0.elapsed_time(e1) / 1e3
        bpack_kernels = bpack.kernels_per_step()
        for b in batches:
            b.step(1, stream.cuda_stream)
        bstatus = [int(b.stats(q)["status"]) for b in batches for q in range(per)]
        del bpack, batches
    finally:
        if old is None:
            os.environ.pop("NSF_PCG_PATH", None)
        else:
            os.environ["NSF_PCG_PATH"] = old
        shutil.rmtree(tmp, ignore_errors=True)
    n = len(steppers)
    return {
        "metric": "config 4b: uneven pack of channel instances on three meshes, aggregate instance-steps/s",
        "value": round(n * K / t_pack, 2), "unit": "instance-steps/s", "n_gpus": 1, "steps": K, "warmup": W,
        "higher_is_better": True, "dtype": "f32-inner/f64-refine",
        "data": "synthetic (seeded DFG channel meshes h=0.025/0.01/0.005; U_max, nu per instance from seed 1)",
        "config": {"workload": f"{per} instances on each of h={hs}, U_max~U[0.2,1.5], nu~logU[5e-4,2e-3], "
                               f"tau={tau}, pressure to 1e-8 rel", "instances": n,
                   "mass_solve": MASS_SOLVES[args.vel_method],
                   "pressure_guess": PRESSURE_GUESSES[args.pressure_guess].format(args.pressure_basis or 250),
                   "mesh_sizes_N_P": {str(h): sizes[h] for h in hs}, "setup_s": round(setup_s, 1),
                   "execution": "one CUDA graph per step whose branches are the 48 instances' steps (nsf_pack); "
                                "cluster-resident solves"},
        "sequential_instance_steps_per_s": round(n * K / t_seq, 2),
        "speedup_vs_sequential": round(t_seq / t_pack, 2),
        "one_instance_alone_steps_per_s": alone,
        "status_all_ok": all(s == 0 for s in status),
        "kernel_launches_total": int(launches),
        "kernels_per_pack_step": int(pack_kernels),
        "batched_pack": {"instance_steps_per_s": round(n * K / t_bpack, 2),
                         "over_pack_of_steppers": round(t_pack / t_bpack, 2),
                         "kernels_per_pack_step": int(bpack_kernels),
                         "status_all_ok": all(s == 0 for s in bstatus),
                         "execution": "the same instances as three nsf_batch objects (one per mesh, same U_max and "
                                      "nu draws) as the branches of one pack graph (nsf_pack_create_batches)"},
    }


def bench_long(args):
    """Config 2 over a long horizon: the h = 0.005 channel of the default workload (U_max = 1.5,
    nu = 1e-3, tau = 1e-4, pressure to 1e-8, mass solves of --vel-method, extrapolated pressure guess) from
    rest for --long-steps steps with the mixed stepper and the FP64 stepper side by side: the
    relative L2 difference of u and p every 1000 steps, and the drag / lift time series (every step,
    written on the device) compared over the whole run.  Both steppers are timed."""
    import numpy as np
    import torch

    import nsfemoptim_gb300 as G

    n, chunk = args.long_steps, 1000
    tmp = tempfile.mkdtemp()
    try:
        mesh = G.load_gmsh(make_mesh(tmp, H, 0))
        ctx = G.build_chorin_context(mesh, PEAK)

        def stepper(prec):
            return G.ChorinStepper(ctx, NU, TAU, precision=prec, vel_method=args.vel_method, vel_max_iters=500, vel_tol=VEL_TOL,
                                   pres_max_iters=5000, pres_tol=PRES_TOL, check_interval=8, use_graph=True,
                                   max_outer=4, inner_tol=1e-5, pressure_guess=args.pressure_guess,
                                   pressure_basis=args.pressure_basis)

        steppers = {"mixed": stepper(G.NSF_PREC_MIXED), "fp64": stepper(G.NSF_PREC_F64)}
        forces = {k: G.Forces(mesh, s) for k, s in steppers.items()}
        series = {k: torch.zeros(n, 2, dtype=torch.float64, device="cuda") for k in steppers}
        stream = torch.cuda.Stream()
        sp = stream.cuda_stream
        secs = {k: 0.0 for k in steppers}
        field = []
        done = 0
        while done < n:
            m = min(chunk, n - done)
            for k, st in steppers.items():
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for i in range(m):
                    st.launch(1, sp)
                    forces[k].into(series[k][done + i], sp)
                e1.record(stream)
                torch.cuda.synchronize()
                secs[k] += e0.elapsed_time(e1) / 1e3
            done += m
            (um, pm), (uf, pf) = steppers["mixed"].state(), steppers["fp64"].state()
            field.append({"step": done, "u_rel_l2": float(np.linalg.norm(um - uf) / np.linalg.norm(uf)),
                          "p_rel_l2": float(np.linalg.norm(pm - pf) / np.linalg.norm(pf))})
        sm, sf = series["mixed"].cpu().numpy(), series["fp64"].cpu().numpy()
        for st in steppers.values():  # one synchronous step each: solver status at the end
            st.step(1, sp)
        ok = all(int(st.stats()["status"]) == 0 for st in steppers.values())
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    fmax = np.abs(sf[:, 0]).max()
    return {
        "metric": "config 2 long run: mixed vs FP64 steppers side by side, field and drag/lift differences",
        "value": round(n / secs["mixed"], 2), "unit": "steps/s", "n_gpus": 1, "steps": n, "higher_is_better": True,
        "dtype": "f32-inner/f64-refine",
        "data": "synthetic (seeded DFG channel mesh, h=0.005)",
        "config": {"workload": f"DFG channel h={H}, Umax=1.5, nu={NU}, tau={TAU}, {n} steps from rest, pressure "
                               f"to {PRES_TOL} rel", "N": ctx.N, "P": ctx.P,
                   "mass_solve": MASS_SOLVES[args.vel_method],
                   "pressure_guess": PRESSURE_GUESSES[args.pressure_guess].format(args.pressure_basis or 250)},
        "fp64_steps_per_s": round(n / secs["fp64"], 2),
        "field_rel_l2_mixed_vs_fp64": field,
        "drag_max_rel_err": float(np.abs(sm[:, 0] - sf[:, 0]).max() / fmax),
        "lift_max_err_rel_to_max_drag": float(np.abs(sm[:, 1] - sf[:, 1]).max() / fmax),
        "drag_fp64_last": float(sf[-1, 0]), "lift_fp64_last": float(sf[-1, 1]),
        "c_drag_fp64_last": float(sf[-1, 0] * 2.0 / ((PEAK / 6.0) ** 2 * 0.1)),  # U_mean = PEAK / 6, D = 0.1
        "status_all_ok": ok,
    }


POISSON_NODES = 1024  # nodes per side of the jittered unit square (1,048,576 nodes)


def bench_poisson(args):
    """Standalone pressure-Poisson solve: P1 Laplacian of a jittered 1024 x 1024-node unit square
    (interior nodes moved by U(+-0.2 h), one diagonal per cell, seed 0), pure Neumann with one
    Dirichlet pin at node 0, RHS i.i.d. N(0,1) from seed 0.  The zero-mean projection of the RHS,
    the pin and the zero-mean shift of the solution run on the device in FP64 (nsf_neumann_*).  FP64
    PCG-SGS against FP32-inner / FP64-refinement, both to 1e-10 relative residual of the pinned
    system; GB/s of the PCG iteration and of the SpMV."""
    import numpy as np
    import scipy.sparse as sp
    import torch

    import nsfemoptim_gb300 as G
    from nsfemoptim_gb300 import meshgen
    from nsfemoptim_gb300.api import HostCsr

    t0 = time.perf_counter()
    mesh = meshgen.jittered_square(POISSON_NODES, seed=0, jitter=0.2)
    rs, ci, val = meshgen.p1_stiffness(mesh.nodes, mesh.triangles)
    full = sp.csr_matrix((val, ci, rs))
    full.sort_indices()
    nfull = full.shape[0]
    fhost = HostCsr(nfull, nfull, full.indptr.astype(np.int32), full.indices.astype(np.int32), full.data)
    a = full[1:, 1:].tocsr()  # the pinned system (for the SpMV timing and the byte counts)
    a.sort_indices()
    n = a.shape[0]
    rng = np.random.default_rng(0)
    bfull = rng.standard_normal(n + 1)
    bproj = bfull - bfull.mean()
    host = HostCsr(n, n, a.indptr.astype(np.int32), a.indices.astype(np.int32), a.data)
    setup_s = time.perf_counter() - t0
    bd = torch.tensor(bfull, device="cuda")

    def ev():
        return torch.cuda.Event(enable_timing=True)

    out = {}
    want = args.poisson_precisions.split(",")
    for name, prec in (("fp64", G.NSF_PREC_F64), ("mixed", G.NSF_PREC_MIXED)):
        if name not in want:
            continue
        s = G.NeumannSolver(fhost, pin=0, precision=prec, max_iters=args.poisson_max_iters, target=1e-10)
        xd = torch.zeros(nfull, dtype=torch.float64, device="cuda")
        best = None
        for rep in range(1 + max(1, args.poisson_reps)):  # the first solve is a warm-up
            xd.zero_()
            torch.cuda.synchronize()
            e0, e1 = ev(), ev()
            e0.record()
            try:
                s.solve(bd, xd)
            except G.NsfError as e:
                if e.status != 3 or args.poisson_max_iters >= 20000:
                    raise  # status 3 (iteration cap) is expected only under a profiling cap
            e1.record()
            torch.cuda.synchronize()
            if rep > 0:
                t = e0.elapsed_time(e1) / 1e3
                best = t if best is None else min(best, t)
        xf = xd.cpu().numpy()
        stt = s.stats()
        its, st = stt["iters"], 0
        # sv: bytes of a value of A p and of the CG vectors, sp: of the SGS sweeps.  The mixed solve
        # of a system this size (cooperative-grid path) is one CG with the FP64 recurrence and A p
        # under the FP32 SGS preconditioner.
        sv, sp = 8, (8 if name == "fp64" else 4)
        nnz = a.nnz
        it_bytes = (nnz * (sv + 4) + (n + 1) * 4 + 2 * n * sv) + \
            2 * ((nnz - n) * (sp + 4) + (n + 1) * 4 + 4 * n * sp) + 7 * n * sv
        out[name] = {"solve_s": round(best, 5), "solves_per_s": round(1.0 / best, 3), "iterations": int(its),
                     "status": int(st),
                     "true_rel_residual": float(np.linalg.norm(bproj - full @ xf) / np.linalg.norm(bproj)),
                     "solution_mean": float(xf.mean()),
                     "us_per_iteration": round(1e6 * best / max(1, its), 3),
                     "pcg_iteration_gbs": round(it_bytes * its / best / 1e9, 1)}
        del s
    # SpMV alone from DRAM: the L2 is flushed before every launch by a 256 MB write followed by a
    # read of the same buffer (the read pass takes the write-backs of the dirty lines, which would
    # otherwise share DRAM with the SpMV).  A 25 us launch bracketed by its own events carries the
    # event and launch gaps, so the time is differential: events around reps x (flush, SpMV) minus
    # events around reps x (flush).
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    flush_sum = torch.zeros((), dtype=torch.float32, device="cuda")
    spmv = {}
    for name, dt, tdt in (("fp64", G.NSF_F64, torch.float64), ("fp32", G.NSF_F32, torch.float32)):
        if not args.poisson_spmv:
            break
        A = G.CsrF.from_host(host, dtype=dt)
        xv = torch.randn(n, dtype=tdt, device="cuda")
        yv = torch.zeros(n, dtype=tdt, device="cuda")
        reps = 20

        def run(with_spmv):
            e0, e1 = ev(), ev()
            torch.cuda.synchronize()
            e0.record()
            for rep in range(reps):
                flush.fill_(float(rep))
                flush_sum.copy_(flush.sum())
                if with_spmv:
                    G.spmv(A, xv, yv)
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / 1e3

        run(True)
        run(False)
        t_both = min(run(True) for _ in range(3))
        t_flush = min(run(False) for _ in range(3))
        t1 = max(t_both - t_flush, 1e-9) / reps
        sv = 8 if name == "fp64" else 4
        byts = a.nnz * (sv + 4) + (n + 1) * 4 + 2 * n * sv
        spmv[name] = {"us": round(1e6 * t1, 2), "gbs": round(byts / t1 / 1e9, 1), "algorithmic_bytes": byts,
                      "timing": f"differential over {reps} (flush, SpMV) pairs"}
    hbm, kind = peaks()
    for v in spmv.values():
        v["frac_of_hbm_peak"] = round(v["gbs"] / hbm, 4)
    return {
        "metric": "config 3: standalone P1 Poisson PCG-SGS to 1e-10 rel (1024x1024 jittered square), solves/s",
        "value": out.get("mixed", out.get("fp64", {})).get("solves_per_s"), "unit": "solves/s", "n_gpus": 1,
        "higher_is_better": True,
        "dtype": "f64 CG recurrence and A p, f32 SGS preconditioner",
        "data": "synthetic (seeded jittered unit square, RHS N(0,1) seed 0)",
        "config": {"workload": "P1 Laplacian, 1024x1024 nodes, jitter 0.2h, one pin", "rows": n, "nnz": int(a.nnz),
                   "setup_s": round(setup_s, 2)},
        "variants": out, "spmv": spmv, "peak": hbm, "peak_kind": kind,
        "mixed_vs_fp64_speedup": (round(out["fp64"]["solve_s"] / out["mixed"]["solve_s"], 3)
                                  if "fp64" in out and "mixed" in out else None),
        "mixed_form": "one CG with the FP64 recurrence, FP64 A p and dot products under the FP32 multicolor SGS "
                      "preconditioner (cooperative grid, one launch), then the FP64 residual test",
    }


def bench_ours(args, rank, world, local_rank):
    import numpy as np
    import torch

    import nsfemoptim_gb300 as G

    torch.cuda.set_device(local_rank)
    tmp = tempfile.mkdtemp()
    try:
        mesh_path = make_mesh(tmp, H, seed=rank)
        t0 = time.perf_counter()
        mesh = G.load_gmsh(mesh_path)
        ctx = G.build_chorin_context(mesh, PEAK)
        setup_s = time.perf_counter() - t0
        N, P, nip = ctx.N, ctx.P, len(ctx.int_p)

        def stepper(precision, graph=True):
            return G.ChorinStepper(ctx, NU, TAU, precision=precision, vel_method=args.vel_method, vel_max_iters=500,
                                   vel_tol=VEL_TOL, pres_max_iters=5000, pres_tol=PRES_TOL, check_interval=8,
                                   use_graph=graph, max_outer=4, inner_tol=1e-5, pressure_guess=args.pressure_guess,
                                   pressure_basis=args.pressure_basis)

        stream = torch.cuda.Stream()
        sp = stream.cuda_stream

        def timed(st, steps, warm):
            """(seconds, kernels launched) for `steps` steps after `warm` untimed ones."""
            with torch.cuda.stream(stream):
                st.step(warm, sp)
                torch.cuda.synchronize()
                if world > 1:
                    torch.distributed.barrier()
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                k0 = G.kernel_launches()
                e0.record(stream)
                st.step(steps, sp)
                e1.record(stream)
                torch.cuda.synchronize()
                k1 = G.kernel_launches()
                if world > 1:
                    torch.distributed.barrier()
                return e0.elapsed_time(e1) / 1e3, k1 - k0

        # ---- main line: mixed precision, graph-captured steps, state resident in HBM
        mixed = stepper(G.NSF_PREC_MIXED)
        clocks = Clocks(local_rank) if rank == 0 else None
        t_mixed, launches = timed(mixed, args.steps, args.warmup)
        clk = clocks.stop() if clocks else None
        st_mixed = mixed.stats()

        # ---- FP64 drop-in on the same workload
        f64 = stepper(G.NSF_PREC_F64)
        t_f64, _ = timed(f64, args.steps, args.warmup)  # the same steps from rest as the main line
        st_f64 = f64.stats()
        u_m, p_m = mixed.state()

        # ---- the literal FP32-inner split (NSF_PREC_MIXED_F32: FastConvection, A u, D u and G p with
        # FP32 values, vectors and sums; FP32 PCG mass (Jacobi) and pressure solves inside FP64
        # refinement / residual replacement) over the same steps from rest, compared with the FP64
        # drop-in after them, beside the main line's split
        f32v = None
        if args.f32_variant:
            u_f, p_f = f64.state()
            v32 = G.ChorinStepper(ctx, NU, TAU, precision=G.NSF_PREC_MIXED_F32, vel_method=2, vel_max_iters=500,
                                  vel_tol=VEL_TOL, pres_max_iters=5000, pres_tol=PRES_TOL, check_interval=8,
                                  use_graph=True, max_outer=4, inner_tol=1e-5, pressure_guess=args.pressure_guess,
                                  pressure_basis=args.pressure_basis)
            t_v, _ = timed(v32, args.steps, args.warmup)
            st_v = v32.stats()
            u_v, p_v = v32.state()
            del v32

            def rel(a, b):
                return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

            f32v = {"steps_per_s": round(world * args.steps / t_v, 3), "ms_per_step": round(1e3 * t_v / args.steps, 4),
                    "stats": st_v, "mass_solve": MASS_SOLVES[2],
                    "after_steps": args.warmup + args.steps,
                    "u_rel_l2_vs_fp64": rel(u_v, u_f), "p_rel_l2_vs_fp64": rel(p_v, p_f),
                    "main_line_u_rel_l2_vs_fp64": rel(u_m, u_f), "main_line_p_rel_l2_vs_fp64": rel(p_m, p_f)}

        # ---- steady-state window: both steppers continue to step --steady-from, then --steady-steps
        # more steps are timed each (the early steps from rest need hundreds of pressure iterations,
        # the developed flow tens)
        steady = None
        if args.steady_steps > 0:
            done = args.warmup + args.steps
            lead = max(0, args.steady_from - done)
            t_sm, _ = timed(mixed, args.steady_steps, lead)
            st_sm = mixed.stats()
            t_sf, _ = timed(f64, args.steady_steps, lead)
            st_sf = f64.stats()
            steady = {"from_step": done + lead, "steps": args.steady_steps,
                      "mixed_steps_per_s": round(args.steady_steps / t_sm, 3),
                      "fp64_steps_per_s": round(args.steady_steps / t_sf, 3),
                      "mixed_over_fp64": round(t_sf / t_sm, 3),
                      "mixed_pres_iters_last": st_sm["pres_iters"], "fp64_pres_iters_last": st_sf["pres_iters"]}
        del f64

        # ---- e2e through the C ABI with host buffers, on a fresh mixed stepper over the same steps
        # from rest as the main line (W untimed, K timed): every step H2D of the state from pinned
        # host memory (set_state, enqueued without waiting), one launched step, D2H of the state to
        # pinned host memory (get_state, which waits for it), all on one stream
        e2e = stepper(G.NSF_PREC_MIXED)
        u_h = torch.zeros(2 * N, dtype=torch.float64, pin_memory=True).numpy()
        p_h = torch.zeros(P, dtype=torch.float64, pin_memory=True).numpy()
        e2e.get_state_into(u_h, p_h, sp)

        def e2e_step():
            # the state continues the run: the pressure-guess history is kept
            e2e.set_state(u_h, p_h, keep_history=True, asynchronous=True, stream=sp)
            e2e.launch(1, sp)
            e2e.get_state_into(u_h, p_h, sp)

        for _ in range(args.warmup):
            e2e_step()
        e2e_steps = args.steps
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step()
        t_e2e = time.perf_counter() - t0
        # the host round trip is exact: after the same W + K steps from rest the state equals the
        # main line's bit for bit
        import numpy as np
        e2e_same = bool(np.array_equal(u_h, u_m) and np.array_equal(p_h, p_m))
        del e2e

        # ---- dominant kernel alone: FastConvection SpMV (I: nnz(K) x 2N) fused with the nu K add
        # (the mixed stepper's kernel: FP32 values of I; u, K, A and the sums as double-floats)
        Ih = ctx.matrix("I")
        Kh = ctx.matrix("K")
        I32 = G.CsrF.from_host(Ih, dtype=G.NSF_F32)
        u2 = G.split_df(torch.tensor(u_m, dtype=torch.float64, device="cuda"))
        K2 = G.split_df(torch.tensor(Kh.values, dtype=torch.float64, device="cuda"))
        A2 = torch.zeros_like(K2)
        reps = 20
        with torch.cuda.stream(stream):
            for _ in range(3):
                G.fastconv_apply_df(I32, K2, NU, u2, A2, sp)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                G.fastconv_apply_df(I32, K2, NU, u2, A2, sp)
            e1.record(stream)
            torch.cuda.synchronize()
        t_fc = e0.elapsed_time(e1) / 1e3 / reps
        nnzI, rowsI = Ih.nnz, Ih.rows
        # values + column indices of I, row starts, u once, K read and A written (8-byte pairs)
        fc_bytes = nnzI * (4 + 4) + (rowsI + 1) * 4 + 2 * N * 8 + 2 * rowsI * 8

        coarse = os.environ.get("NSF_PRES_COARSE", "1") != "0"
        pcg_form = ("coarse" if coarse else
                    "classic" if os.environ.get("NSF_PCG_FORM") == "classic" else "eisenstat")
        xy_int = mesh.pressure_xy()[ctx.int_p]
        # ---- dominant kernel: the cluster-resident pressure PCG (FP32 inner solve of the
        # refinement).  Per-iteration time from two solves that differ only in the iteration cap
        # (same launches, same setup), each solve bracketed by CUDA events on its stream.
        Kpi = ctx.matrix("Kpi")
        gen = torch.Generator(device="cuda").manual_seed(1)
        bP = torch.randn(Kpi.rows, dtype=torch.float64, device="cuda", generator=gen)
        pcg_t = {}
        for cap in (20, 80):
            s = G.create_solver("pcg", 1, Kpi, cap, 1e-30, 1000, precision=G.NSF_PREC_MIXED)
            if coarse:  # the stepper's pressure solve: the two-level preconditioner on mesh cells
                s.setCoarse(xy_int, int(os.environ.get("NSF_PRES_COARSE_ROWS", "240")))
            s.getRhs().copy_(bP)
            best = None
            for rep in range(4):
                s.getSol().zero_()
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                s.solve()
                e1.record()
                torch.cuda.synchronize()
                dt = e0.elapsed_time(e1) / 1e3
                if rep > 0:
                    best = dt if best is None else min(best, dt)
            pcg_t[cap] = (best, s.getLastIterations())
            del s
        t_it = (pcg_t[80][0] - pcg_t[20][0]) / max(1, pcg_t[80][1] - pcg_t[20][1])
        n_p, nnz_p = Kpi.rows, Kpi.nnz
        if pcg_form in ("classic", "coarse"):
            # algorithmic bytes of one classical PCG iteration in FP32 (sv = si = 4): SpMV + two SGS
            # sweeps + 7 vector passes, rows/nnz of the internal pressure system; the coarse
            # correction adds the restriction (r read), the corrected z (z read, z' written) and its
            # gather in the SpMV (the coarse inverse lives in shared memory)
            spmv_b = nnz_p * 8 + (n_p + 1) * 4 + 2 * n_p * 4
            sweep_b = (nnz_p - n_p) * 8 + (n_p + 1) * 4 + 3 * n_p * 4 + n_p * 4
            pcg_bytes = spmv_b + 2 * sweep_b + 7 * n_p * 4 + (3 * n_p * 4 if pcg_form == "coarse" else 0)
        else:
            # Eisenstat's form: every off-diagonal entry once (backward sweep over the later-colour
            # entries, forward sweep over the earlier-colour ones), the row structure twice, 22
            # vector passes (update: p, s, x~, r~, w, d read and p, s, x~, r~ written; backward: r~,
            # 1/d read, t written, t gathered; forward: r~, t, 1/d, d read, f, w written, f and r~
            # gathered)
            pcg_bytes = (nnz_p - n_p) * 8 + 2 * (n_p + 1) * 4 + 22 * n_p * 4

        # ---- the double-float Chebyshev iteration of the mass solves (with the two-level pressure
        # solve the largest share of the step): per-iteration time from two mass solves whose a priori
        # counts differ (tolerances 1e-8 and 1e-4), each bracketed by CUDA events; algorithmic bytes
        # of one iteration: M's SELL entries (double-float value + column), the slice starts, and
        # d gathered once, x and r read and written, d' written (2N double-floats each), perm and
        # D^-1 (N each)
        cheb = None
        if args.vel_method == 3:
            ms = stepper(G.NSF_PREC_MIXED)
            bM = torch.randn(2 * N, dtype=torch.float64, device="cuda", generator=gen)
            xM = torch.zeros_like(bM)
            ct = {}
            for tol in (1e-8, 1e-4):
                best, its = None, 0
                for rep in range(4):
                    torch.cuda.synchronize()
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    its = ms.mass_solve(bM, xM, tol, sp)
                    e1.record(stream)
                    torch.cuda.synchronize()
                    dt = e0.elapsed_time(e1) / 1e3
                    if rep > 0:
                        best = dt if best is None else min(best, dt)
                ct[tol] = (best, its)
            t_ch = (ct[1e-8][0] - ct[1e-4][0]) / max(1, ct[1e-8][1] - ct[1e-4][1])
            mnnz = ctx.matrix("M").nnz
            ch_bytes = mnnz * (8 + 4) + (N // 32 + 1) * 4 + 2 * N * 8 * 6 + N * (8 + 4)
            cheb = {"bound": "hbm", "kernel": "kChebStepDfSplit (mass solves: one double-float Chebyshev "
                                              "iteration, a warp per SELL slice and channel)",
                    "achieved": round(ch_bytes / t_ch / 1e9, 1), "unit": "GB/s",
                    "algorithmic_bytes_per_iteration": ch_bytes, "iteration_us": round(t_ch * 1e6, 3),
                    "note": "M, its SELL copy and the vectors (~40 MB at h = 0.005) stay in L2 between "
                            "iterations, so the rate can exceed what DRAM alone would give"}
            del ms

        # ---- accuracy (untimed): mixed vs FP64 fields and drag/lift series from rest
        accuracy, f64_step4 = (accuracy_run(G, ctx, mesh, stepper, torch, stream) if args.accuracy
                               else (None, None))

        times = [t_mixed]
        if world > 1:
            tt = torch.tensor([t_mixed, t_f64, t_e2e], dtype=torch.float64, device="cuda")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            t_mixed, t_f64, t_e2e = tt.tolist()
        if rank != 0:
            return None

        hbm, kind = peaks()
        achieved = fc_bytes / t_fc / 1e9
        achieved_pcg = pcg_bytes / t_it / 1e9
        pcg_line = {"bound": "hbm",
                    "kernel": {"classic": "kPcgClusterDs<float,1> (pressure PCG-SGS, FP32, classical form)",
                               "coarse": "kPcgClusterDs<float,1,CO> (pressure PCG, FP32, multicolor SGS plus the "
                                         "coarse correction on mesh cells, classical form)",
                               "eisenstat": "kPcgClusterEis<float,1> (pressure PCG-SGS, FP32, Eisenstat's form, one "
                                            "reduction per iteration)"}[pcg_form],
                    "achieved": round(achieved_pcg, 1), "peak": hbm, "unit": "GB/s",
                    "frac": round(achieved_pcg / hbm, 4), "peak_kind": kind,
                    "algorithmic_bytes_per_iteration": pcg_bytes, "iteration_us": round(t_it * 1e6, 3),
                    "traffic": None,
                    "note": "vectors and matrix live in shared memory across the cluster; the kernel is bound by "
                            "barrier/gather latency, not HBM (ncu DRAM traffic per launch is ~1% of the "
                            "algorithmic bytes)"}
        if cheb is not None:
            cheb.update({"peak": hbm, "frac": round(cheb["achieved"] / hbm, 4), "peak_kind": kind, "traffic": None})
        steps_s = world * args.steps / t_mixed
        line = {
            "metric": METRIC,
            "value": round(steps_s, 3),
            "unit": "steps/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(1e3 * t_mixed / args.steps, 4),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32/df32-inner, f64-refine",
            "data": "synthetic (seeded DFG channel mesh, h=0.005)",
            "config": {"workload": "DFG channel h=0.005, Umax=1.5, nu=1e-3, tau=1e-4, P2/P1, "
                                   "pressure PCG-SGS to 1e-8 rel", "triangles": mesh.num_tri, "N": N, "P": P,
                       "internal_pressure": nip, "nnz_I": nnzI, "parallelism": f"replicas x{world}",
                       "l2": "working set > L2 (FastConvection matrix %.0f MB FP32)" % (nnzI * 8 / 1e6),
                       "graph": True, "setup_s": round(setup_s, 2),
                       "mass_solve": MASS_SOLVES[args.vel_method],
                       "pressure_guess": PRESSURE_GUESSES[args.pressure_guess].format(args.pressure_basis or 250)},
            "e2e": {"value": round(world * e2e_steps / t_e2e, 3), "unit": "steps/s",
                    "h2d_bytes_per_step": (2 * N + P) * 8, "d2h_bytes_per_step": (2 * N + P) * 8,
                    "path": "per step, on one stream: set_state (u, p from pinned host memory, renumbered on "
                            "the device, enqueued without waiting; the run's pressure-guess history kept), one "
                            "graph-launched step, get_state (u, p to pinned host memory; the one wait per step)",
                    "state_equals_value_run": e2e_same},
            "gpu_launches": int(launches),
            "roofline": cheb if cheb is not None else pcg_line,
            "roofline_pressure": pcg_line if cheb is not None else None,
            "roofline_fastconv": {"bound": "hbm", "kernel": "kFastConvSellDf (A = nu K + I u, FP32 I values; u, K, A and sums as "
                                                "double-floats, SELL-32-256)",
                                  "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                                  "frac": round(achieved / hbm, 4), "peak_kind": kind,
                                  "algorithmic_bytes": fc_bytes, "launch_us": round(t_fc * 1e6, 2)},
            "variants": {"fp64": {"steps_per_s": round(world * args.steps / t_f64, 3),
                                  "ms_per_step": round(1e3 * t_f64 / args.steps, 4),
                                  "stats": st_f64},
                         "mixed_over_fp64": round(t_f64 / t_mixed, 3),
                         "mixed_stats": st_mixed,
                         "steady": steady,
                         "mixed_f32_inner": f32v},
            "precision_split": ("FP32 operator values and FP32 inner CG (pressure: FP64 residual replacement); "
                                "FastConvection, A u and the Chebyshev mass solves in double-float (float pairs on "
                                "the FP32 pipes, ~48 bits); D u and G p with FP64 sums; state, residuals and step "
                                "lengths FP64. variants.mixed_f32_inner is the literal FP32-inner split"),
        }
        if accuracy is not None:
            line["accuracy"] = accuracy
            line["_f64_step4"] = f64_step4  # compared with the oracle in main(), then dropped
        if clk:
            line["clocks"] = clk
        return line
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-sample-steps", type=int, default=-1,
                    help="CPU baseline of the channel workload: -1 the timed GPU window (--warmup steps from "
                         "rest, then --steps timed), k > 0 the first k steps after one warm-up, 0 none")
    ap.add_argument("--steady-from", type=int, default=500,
                    help="channel workload: step from rest at which the steady-state window starts")
    ap.add_argument("--steady-steps", type=int, default=100,
                    help="channel workload: steps timed in the steady-state window (0: none)")
    ap.add_argument("--no-accuracy", dest="accuracy", action="store_false",
                    help="skip the untimed mixed-vs-FP64 field and drag/lift comparison")
    ap.add_argument("--workload", default="channel", choices=["channel", "poisson", "small", "batch", "pack", "adjoint", "long"],
                    help="channel: the h=0.005 time step (default); poisson: the standalone 1M-DOF pressure "
                         "solve; small: the plain FP64 h=0.02 channel; batch: 64 instances at h=0.01; "
                         "adjoint: the drag gradient at h=0.01 over 1000 steps")
    ap.add_argument("--vel-method", type=int, default=3, choices=[1, 2, 3, 4],
                    help="channel, batch, pack and long workloads: mass solve, 1 PCG multicolor SGS, 2 PCG "
                         "Jacobi, 3 Chebyshev Jacobi, 4 the same warm-started from the previous step")
    ap.add_argument("--pressure-basis", type=int, default=0,
                    help="pressure guess 2: basis vectors (3..256; 0: 250)")
    ap.add_argument("--pressure-guess", type=int, default=2, choices=[0, 1, 2],
                    help="channel, batch, pack and long workloads: pressure initial guess, 0 previous "
                         "solution, 1 extrapolated, 2 projected onto earlier solutions")
    ap.add_argument("--adjoint-steps", type=int, default=1000)
    ap.add_argument("--adjoint-checkpoint", type=int, default=50)
    ap.add_argument("--adjoint-snapshots", type=int, default=20,
                    help="adjoint workload: stored states of the binomial-checkpointing variant")
    ap.add_argument("--adjoint-precision", default="mixedsolve", choices=["f64", "mixedsolve"])
    ap.add_argument("--adjoint-vel-method", type=int, default=2, choices=[1, 2, 3],
                    help="mass solve: 1 PCG multicolor SGS, 2 PCG Jacobi, 3 Chebyshev Jacobi")
    ap.add_argument("--adjoint-reps", type=int, default=1, help="timed gradient evaluations")
    ap.add_argument("--adjoint-warmup", type=int, default=1, help="untimed gradient evaluations")
    ap.add_argument("--adjoint-cpu-steps", type=int, default=6)
    ap.add_argument("--adjoint-fd-coefs", type=int, nargs="*", default=[1],
                    help="inflow coefficients (1..16) checked by central differences besides nu")
    ap.add_argument("--no-adjoint-variants", dest="adjoint_variants", action="store_false")
    ap.add_argument("--no-adjoint-fd", dest="adjoint_fd", action="store_false",
                    help="skip the central-difference check")
    ap.add_argument("--small-steps", type=int, default=2000)
    ap.add_argument("--small-cpu-steps", type=int, default=100)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=20)
    ap.add_argument("--pack-per-mesh", type=int, default=16, help="pack workload: instances per mesh")
    ap.add_argument("--pack-steps", type=int, default=20)
    ap.add_argument("--long-steps", type=int, default=10000, help="long workload: steps from rest")
    ap.add_argument("--poisson-reps", type=int, default=2)
    ap.add_argument("--f32-variant", type=int, default=1,
                    help="channel workload: also time the literal FP32-inner split (NSF_PREC_MIXED_F32)")
    ap.add_argument("--poisson-max-iters", type=int, default=20000,
                    help="poisson workload: iteration cap of each solve (a small cap gives short launches to profile)")
    ap.add_argument("--poisson-precisions", default="fp64,mixed", help="poisson workload: solves to run")
    ap.add_argument("--poisson-spmv", type=int, default=1, help="poisson workload: 0 skips the SpMV timing")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.workload == "adjoint" and args.impl == "reference":
        if rank != 0:
            return
        import numpy as np
        tmp = tempfile.mkdtemp()
        try:
            path = make_mesh(tmp, ADJ_H, 0)
            import oracle
            oracle.build()
            om = oracle.Mesh(path)
            oc = oracle.Context(om, ADJ_PEAK, True)
            xy = om.v_xy.astype(np.float64)[oc.dir_ids]
            inflow = np.abs(xy[:, 0]) < 1e-9
            basis = np.where(inflow[:, None], np.sin(np.pi * np.outer(xy[:, 1], np.arange(1, 17)) / 0.41), 0.0)
            theta = 0.01 * np.random.default_rng(0).standard_normal(16)
            k = max(1, args.adjoint_cpu_steps)
            cpu_t, _, _, _ = _adjoint_oracle_sample(path, k, theta, basis, oc.dir_vx.copy(),
                                                    2.0 / ((ADJ_PEAK / 6.0) ** 2 * 0.1))
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
        v = round(cpu_t * args.adjoint_steps / k, 1)
        print(json.dumps({"impl": "reference", "metric": ADJ_METRIC, "value": v, "unit": "s", "n_gpus": 0,
                          "steps": 1, "warmup": 0, "higher_is_better": False, "dtype": "f64",
                          "config": {"workload": "adjoint drag gradient, DFG channel h=0.01, 1000 steps"},
                          "cpu_baseline": {"value": v, "unit": "s", "cores": CPU_THREADS, "kind": "port",
                                           "sample": f"FP64 C oracle forward + adjoint over {k} steps on {CPU_THREADS} "
                                                     f"host threads, scaled to {args.adjoint_steps}"},
                          "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return

    if args.workload in ("poisson", "small", "batch", "pack", "adjoint", "long"):
        if rank == 0 and args.impl == "ours":
            fn = {"poisson": bench_poisson, "small": bench_small, "batch": bench_batch,
                  "pack": bench_pack, "adjoint": bench_adjoint, "long": bench_long}[args.workload]
            print(json.dumps(fn(args)))
        return

    if args.impl == "reference":
        if rank != 0:
            return
        tmp = tempfile.mkdtemp()
        try:
            path = make_mesh(tmp, H, 0)
            k, w = max(1, min(args.steps, 400)), args.warmup
            sps, dt, ctx, _ = run_cpu_reference(path, k, w)
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
        line = {"impl": "reference", "metric": METRIC, "value": round(sps, 4), "unit": "steps/s", "n_gpus": 0,
                "steps": k, "warmup": w, "ms_per_step": round(1e3 * dt / k, 2),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded DFG channel mesh, h=0.005)",
                "config": {"workload": "DFG channel h=0.005, Umax=1.5, nu=1e-3, tau=1e-4, P2/P1, "
                                       "pressure PCG-SGS to 1e-8 rel", "N": ctx.N, "P": ctx.P},
                "cpu_baseline": {"value": round(sps, 4), "unit": "steps/s", "cores": CPU_THREADS, "kind": "port",
                                 "sample": f"time steps {w + 1}..{w + k} from rest (after {w} warm-up steps), the "
                                           f"reference's algorithm (mass and pressure PCG with the multicolor SGS "
                                           f"preconditioner, previous-solution pressure guess), FP64 C oracle on "
                                           f"{CPU_THREADS} host threads"},
                "e2e": {"value": round(sps, 4), "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    line = bench_ours(args, rank, world, local_rank)
    if rank == 0 and line is not None:
        f64_step4 = line.pop("_f64_step4", None)
        # CPU baseline on a bounded sample of the same workload (rank 0, N = 1 only)
        if world == 1 and args.cpu_sample_steps != 0:
            cw, ck = (args.warmup, args.steps) if args.cpu_sample_steps < 0 else (1, args.cpu_sample_steps)
            tmp = tempfile.mkdtemp()
            try:
                path = make_mesh(tmp, H, 0)
                sps, dt, _, snap = run_cpu_reference(path, ck, cw, args.vel_method, args.pressure_guess,
                                                     args.pressure_basis, snapshot_step=4)
                uo, po, fo = snap
                line["cpu_baseline"] = {"value": round(sps, 4), "unit": "steps/s", "cores": CPU_THREADS, "kind": "port",
                                        "sample": f"time steps {cw + 1}..{cw + ck} from rest (after {cw} warm-up "
                                                  f"steps) of the same workload and algorithm, FP64 C oracle on "
                                                  f"{CPU_THREADS} host threads (OpenMP)"}
                if f64_step4 is not None and cw + ck >= 4:
                    # the oracle has run 4 steps from rest: the FP64 GPU state after 4 steps vs it
                    import numpy as np
                    ug, pg, fg = f64_step4
                    line["accuracy"]["fp64_vs_oracle_step4"] = {
                        "u_rel_l2": float(np.linalg.norm(ug - uo) / np.linalg.norm(uo)),
                        "p_rel_l2": float(np.linalg.norm(pg - po) / np.linalg.norm(po)),
                        "drag_rel_err": float(abs(fg[0] - fo[0]) / abs(fo[0])),
                        "lift_err_rel_to_drag": float(abs(fg[1] - fo[1]) / abs(fo[0]))}
            finally:
                shutil.rmtree(tmp, ignore_errors=True)
        print(json.dumps(line))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
