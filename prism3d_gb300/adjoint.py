"""Differentiable steady state: torch.autograd.Function over the GB300
solver and its hand-written adjoint.

    problem = SteadyProblem(density, box_size, G0_external, ...)
    theta = torch.zeros(9, dtype=torch.float64, requires_grad=True)
    loss = SteadyStateLoss.apply(theta, problem)     # forward: full solve
    loss.backward()                                  # adjoint sweeps
    theta.grad                                       # dL/dtheta

theta[0:8] are log multipliers of the reduced network's rate coefficients
(PDRSolverGPU.RATE_NAMES), theta[8] the log of the external-field scale
(G0).  The loss is sum over cells of n_H dx sum_s w_columns[s] x_s -- weighted
column sums along x over the whole grid, species x_HI, x_H2, x_C+, x_C,
x_CO -- plus w_T * mean(T_gas), at the converged steady state.  With
``T_fixed`` (an array) the temperature is an input held at those values and
only chemistry and shielding are solved.
"""
from __future__ import annotations

import numpy as np
import torch

from .solver import PDRSolverGPU


class SteadyProblem:
    """A density grid and solver settings; holds one solver per G0 scale."""

    def __init__(self, density, box_size, G0_external, zeta_CR_0=2e-16, nside_rt=1,
                 T_init=100.0, tol=1e-11, n_allow=64, max_iterations=20000, mixed=False,
                 w_chem=0.1, w_columns=(0.0, 0.0, 1.0, 1.0, 1.0), w_T=1.0, T_fixed=None,
                 adjoint_tol=1e-10):
        self.args = (density, box_size)
        self.G0 = np.atleast_1d(np.asarray(G0_external, float))
        self.kw = dict(zeta_CR_0=zeta_CR_0, nside_rt=nside_rt, T_init=T_init)
        self.tol, self.max_iterations, self.mixed, self.w_chem = tol, max_iterations, mixed, w_chem
        self.n_allow = n_allow
        self.w_columns = np.asarray(w_columns, float)
        self.w_T = float(w_T)
        self.T_fixed = None if T_fixed is None else np.asarray(T_fixed, float)
        self.adjoint_tol = adjoint_tol
        self._solver = None
        self._g0_scale = None
        self._theta = None  # parameters of the solver's current state

    def solve(self, theta):
        """Converged solver at parameters theta (9)."""
        theta = np.asarray(theta, float)
        if self._theta is not None and np.array_equal(theta, self._theta):
            return self._solver
        gs = float(np.exp(theta[8]))
        if self._solver is None or self._g0_scale != gs:
            if self._solver is not None:
                self._solver.close()
            self._solver = PDRSolverGPU(*self.args, G0_external=self.G0 * gs, **self.kw)
            self._g0_scale = gs
        s = self._solver
        s.set_rate_scale(np.exp(theta[:8]))
        s.reset()
        if self.T_fixed is not None:
            s.set("T_gas", self.T_fixed)
            s.set_fixed_temperature(True)
        ok = s.run(max_iterations=self.max_iterations, convergence_tol=self.tol,
                   mixed=self.mixed, w_chem=self.w_chem, n_allow=self.n_allow)
        if not ok:
            self._theta = None
            raise RuntimeError(f"steady state not converged (last change {s.last_change:.3e})")
        self._theta = theta.copy()
        return s

    def loss(self, s):
        cols = (s.x_HI, s.x_H2, s.x_Cp, s.x_C, s.x_CO)
        col = sum(float(np.sum(s.density * s.cell_size * w * x))
                  for w, x in zip(self.w_columns, cols) if w != 0.0)
        return col + self.w_T * float(np.mean(s.T_gas))

    def gradient(self, theta):
        s = self.solve(theta)
        r = s.adjoint(w_columns=self.w_columns, w_T=self.w_T, tol=self.adjoint_tol)
        if not r["converged"]:
            raise RuntimeError(r["message"])
        return r["grad"]

    def close(self):
        if self._solver is not None:
            self._solver.close()
            self._solver = None
        self._theta = None


class SteadyStateLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, problem):
        th = theta.detach().cpu().numpy().astype(np.float64)
        s = problem.solve(th)
        ctx.problem = problem
        ctx.th = th
        return torch.tensor(problem.loss(s), dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        g = torch.from_numpy(ctx.problem.gradient(ctx.th))
        return g * grad_out.detach().cpu().to(torch.float64), None
