"""Gradient-check harness of the discrete adjoint: the drag functional of a channel run as a
``torch.autograd.Function`` of the viscosity and the coefficients of a sine-series perturbation of
the inflow profile.  ``forward`` is a plain forward run of the FP64 stepper (nothing is recorded);
``backward`` runs the adjoint (``nsf_adjoint_run``) at the saved inputs.  So
``torch.autograd.gradcheck`` compares the adjoint with FP64 central finite differences of the very
same discrete forward map.  The product API is the C ABI (``Adjoint``); this wrapper exists only for
gradient checks.

The functional: J = sum_n w[n] c_D(u_n, p_n), c_D = 2 F_x / (U_mean^2 D) the drag coefficient of the
cylinder (D = 0.1; the context's inflow is peak * y (H - y) / H^2, so U_max = peak / 4 and
U_mean = 2/3 U_max = peak / 6), u_n, p_n the state after step n,
starting from rest with the perturbed inflow imposed.  The inflow x values are
g(y) = g0(y) + sum_k theta_k sin(k pi y / H) on the nodes at x = 0 (H = 0.41), g0 the parabolic
profile of the context (the reference's, cpp/execs/NavierStokes/src/buildContext.cpp:64-93).
"""

from __future__ import annotations

import numpy as np
import torch

from .api import NSF_PREC_F64, Adjoint, ChorinContext, ChorinStepper, Forces, Mesh

H_CHANNEL = 0.41
D_CYLINDER = 0.1


class DragProblem:
    """One channel problem: mesh, context, an FP64 stepper, its force functional and adjoint."""

    def __init__(self, mesh: Mesh, ctx: ChorinContext, peak: float, nu: float, tau: float, n_steps: int,
                 weights, n_coef: int = 16, tol: float = 1e-13, checkpoint_interval: int = 50,
                 max_iters: int = 20000, precision: int = NSF_PREC_F64, max_outer: int = 6,
                 inner_tol: float = 1e-5, vel_method: int = 1, snapshots: int = 0):
        """precision: NSF_PREC_F64 (FP64 solves) or NSF_PREC_F64_MIXEDSOLVE (FP64 operators, FP32 CG
        inside FP64 refinement / residual replacement to the same tolerance; max_outer passes with
        inner tolerance inner_tol).  vel_method: mass solve, 1 PCG-SGS, 2 PCG-Jacobi, 3 Chebyshev-Jacobi.
        snapshots > 0: binomial checkpointing with that many stored states (checkpoint_interval ignored)."""
        self.mesh, self.ctx = mesh, ctx
        self.n_steps = int(n_steps)
        self.stepper = ChorinStepper(ctx, nu, tau, precision=precision, vel_method=vel_method,
                                     vel_max_iters=max_iters,
                                     vel_tol=tol, pres_max_iters=max_iters, pres_tol=tol, use_graph=True,
                                     max_outer=max_outer, inner_tol=inner_tol)
        self.forces = Forces(mesh, self.stepper)
        self.adjoint = Adjoint(self.stepper, self.forces, checkpoint_interval=checkpoint_interval,
                               max_iters=max_iters, tol=tol, snapshots=snapshots)
        u_mean = peak / 6.0
        self.scale = 2.0 / (u_mean * u_mean * D_CYLINDER)
        self.w = np.ascontiguousarray(np.broadcast_to(np.asarray(weights, np.float64), (self.n_steps,))) * self.scale
        xy = mesh.arrays()[2].astype(np.float64)[ctx.dir_ids]
        inflow = np.abs(xy[:, 0]) < 1e-9
        k = np.arange(1, n_coef + 1)
        self.basis = np.where(inflow[:, None], np.sin(np.pi * np.outer(xy[:, 1], k) / H_CHANNEL), 0.0)
        self.g0 = ctx.dir_vx.copy()
        self.N, self.P = ctx.N, ctx.P
        # a stream of its own: the default stream's handle is 0, which the C ABI reads as "the
        # stepper's stream", a non-blocking stream the default stream does not wait for
        self._stream = torch.cuda.Stream()
        self._dev = torch.zeros(max(1, self.n_steps), 2, dtype=torch.float64, device="cuda")

    def _reset(self, nu: float, theta: np.ndarray):
        self.stepper.set_nu(nu)
        self.stepper.set_state(np.zeros(2 * self.N), np.zeros(self.P))
        self.stepper.set_dirichlet(self.g0 + self.basis @ theta)

    def value(self, nu: float, theta) -> float:
        """J from a forward run alone (graph replays; forces written on the device)."""
        theta = np.asarray(theta, np.float64)
        self._reset(nu, theta)  # synchronous
        torch.cuda.current_stream().synchronize()
        with torch.cuda.stream(self._stream):
            stream = self._stream.cuda_stream
            self._dev.zero_()
            for n in range(self.n_steps):
                self.stepper.launch(1, stream)
                if self.w[n] != 0.0:
                    self.forces.into(self._dev[n], stream)
            f = self._dev[:self.n_steps, 0].cpu().numpy()
        self._stream.synchronize()
        return float(np.dot(self.w, f))

    def gradient(self, nu: float, theta):
        """(J, dJ/dnu, dJ/dtheta, dJ/d dirVx) from the adjoint."""
        theta = np.asarray(theta, np.float64)
        self._reset(nu, theta)
        J, gnu, gdir, _ = self.adjoint.run(self.n_steps, self.w)
        return J, gnu, self.basis.T @ gdir, gdir


class DragFunction(torch.autograd.Function):
    """J(nu, theta) of a DragProblem (nu: 1-element tensor, theta: K coefficients);
    backward = the discrete adjoint."""

    @staticmethod
    def forward(ctx, nu: torch.Tensor, theta: torch.Tensor, problem: DragProblem):
        ctx.problem = problem
        nu_v = float(nu.detach().reshape(-1)[0])
        th = theta.detach().cpu().numpy().copy()
        ctx.point = (nu_v, th)
        return torch.tensor(problem.value(nu_v, th), dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        nu_v, th = ctx.point
        _, gnu, gth, _ = ctx.problem.gradient(nu_v, th)
        g = float(gJ)
        return (torch.full((1,), g * gnu, dtype=torch.float64), torch.from_numpy(g * gth).to(torch.float64), None)


def drag(problem: DragProblem, nu: torch.Tensor, theta: torch.Tensor) -> torch.Tensor:
    return DragFunction.apply(nu, theta, problem)
