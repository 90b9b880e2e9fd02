"""Adjoint of the steady state against central finite differences (GPU).

Grid: the 16^3 log-normal cube (mean n_H 1e4, sigma_ln 1.0, G0 1e4 on -x,
12 rays).  Parameters: log multipliers of the eight reduced-network rate
coefficients and log G0.  Losses: the C+, CO and H2 columns summed over the
grid and the mean T_gas.  The forward solves are FP64 to a relative change of
1e-11 (at most 8 cells above); the finite differences use a step of 1e-5 in
log space (1e-4 and 1e-6 give the same values to the digits compared).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = 1e-5
LOSSES = {"CO": ((0, 0, 0, 0, 1), 0.0), "C+": ((0, 0, 1, 0, 0), 0.0),
          "H2": ((0, 1, 0, 0, 0), 0.0), "T": ((0, 0, 0, 0, 0), 1.0)}


def _loss(s, w, wt):
    cols = (s.x_HI, s.x_H2, s.x_Cp, s.x_C, s.x_CO)
    return (sum(float(np.sum(s.density * s.cell_size * a * x)) for a, x in zip(w, cols) if a)
            + wt * float(np.mean(s.T_gas)))


def _problem(T_fixed=None):
    from prism3d_gb300 import fields
    from prism3d_gb300.adjoint import SteadyProblem
    dens, g0, nside, zeta, cell = fields.workload("cube16", seed=1)
    return SteadyProblem(dens, cell * dens.shape[0], g0, zeta_CR_0=zeta, nside_rt=nside,
                         tol=1e-11, n_allow=8, max_iterations=6000, T_fixed=T_fixed)


def _fd_check(P, names):
    th0 = np.zeros(9)
    s = P.solve(th0)
    adj = {}
    for k in names:
        w, wt = LOSSES[k]
        r = s.adjoint(w_columns=w, w_T=wt)
        assert r["converged"], r["message"]
        adj[k] = r["grad"]
    fd = {k: np.zeros(9) for k in names}
    for j in range(9):
        e = np.zeros(9)
        e[j] = H
        vals = []
        for sg in (1, -1):
            sp = P.solve(th0 + sg * e)
            vals.append({k: _loss(sp, *LOSSES[k]) for k in names})
        for k in names:
            fd[k][j] = (vals[0][k] - vals[1][k]) / (2 * H)
    for k in names:
        g, f = adj[k], fd[k]
        scale = np.max(np.abs(f))
        assert scale > 0
        assert np.max(np.abs(g - f)) <= 1e-4 * scale, (k, g, f)
        big = np.abs(f) > 1e-2 * scale
        assert np.all(np.abs(g - f)[big] <= 1e-4 * np.abs(f)[big]), (k, g, f)
    return adj


def test_adjoint_matches_finite_differences_thermal():
    P = _problem()
    try:
        _fd_check(P, ["CO", "C+", "H2", "T"])
    finally:
        P.close()


def test_adjoint_matches_finite_differences_fixed_temperature():
    P0 = _problem()
    T = P0.solve(np.zeros(9)).T_gas.copy()
    P0.close()
    P = _problem(T_fixed=T)
    try:
        _fd_check(P, ["CO", "C+", "H2"])
    finally:
        P.close()


def test_autograd_function():
    torch = pytest.importorskip("torch")
    from prism3d_gb300.adjoint import SteadyStateLoss
    P = _problem()
    P.w_columns = np.array([0.0, 0.0, 0.0, 0.0, 1e-20])
    P.w_T = 1.0
    try:
        theta = torch.zeros(9, dtype=torch.float64, requires_grad=True)
        loss = SteadyStateLoss.apply(theta, P)
        loss.backward()
        s = P.solve(np.zeros(9))
        assert abs(loss.item() - P.loss(s)) <= 1e-12 * abs(loss.item())
        r = s.adjoint(w_columns=P.w_columns, w_T=1.0)
        np.testing.assert_allclose(theta.grad.numpy(), r["grad"], rtol=1e-12, atol=0)
    finally:
        P.close()


def test_density_gradient_matches_finite_differences():
    """d/d log n_H of single cells: own residual, column layers downstream
    and the ray march (G0 over all rays, A_V / N_H over the selected one)."""
    from prism3d_gb300 import fields
    from prism3d_gb300.adjoint import SteadyProblem
    dens, g0, nside, zeta, cell = fields.workload("cube16", seed=1)
    nx = dens.shape[0]

    def problem(D):
        return SteadyProblem(D, cell * nx, g0, zeta_CR_0=zeta, nside_rt=nside, tol=1e-11,
                             n_allow=8, max_iterations=6000)

    P = problem(dens)
    s = P.solve(np.zeros(9))
    names = ["H2", "T"]
    adj = {k: s.adjoint(w_columns=LOSSES[k][0], w_T=LOSSES[k][1],
                        density_gradient=True)["grad_ln_nH"] for k in names}
    P.close()
    for c in [(0, 8, 8), (3, 2, 12), (9, 7, 4), (2, 11, 11)]:
        vals = []
        for sg in (1, -1):
            D = dens.copy()
            D[c] *= np.exp(sg * H)
            Q = problem(D)
            sp = Q.solve(np.zeros(9))
            vals.append({k: _loss(sp, *LOSSES[k]) for k in names})
            Q.close()
        for k in names:
            fd = (vals[0][k] - vals[1][k]) / (2 * H)
            g = adj[k][c]
            assert abs(g - fd) <= 1e-4 * np.max(np.abs(adj[k])) + 1e-3 * abs(fd), (k, c, g, fd)
