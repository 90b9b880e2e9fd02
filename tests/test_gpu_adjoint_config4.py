"""Adjoint gradients on the 32^3 cube of the adjoint benchmark configuration
(log-normal, mean n_H 3e4, sigma_ln 1.0, G0 1e4 on -x, 12 rays), checked on
50 seeded parameter draws against central finite differences (GPU).

Draws: the nine global parameters (log multipliers of the eight reduced-
network rate coefficients, log G0) and 41 seeded cells' log n_H.  Loss: the
C+ and CO columns summed over the grid.  (The sum of the C+, C and CO
columns is constant: the reduced network conserves carbon.)  Temperature is
held at the converged FP64 state's T_gas: at this size the thermally coupled
FP64 solves at moved parameters do not settle in a few bistable cells (a
cell keeps switching thermal branch by ~1% per iteration), so no
finite-difference reference exists for that coupling here; the thermally
coupled adjoint is checked on the 16^3 cube (tests/test_gpu_adjoint.py).

Step: 1e-5 in log space.  With the step of 1e-4 one cell of this grid
changes chemical branch between the two perturbed solves (its x_CO moves by
5 orders of magnitude at log G0 + 1e-4), so that quotient is not a
derivative; at 1e-5 and 1e-6 the quotients agree with each other and with
the adjoint.  Tolerance: 1e-4 of the largest finite difference, and 1e-3
relative where a component is above 1e-2 of it.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = 1e-5
W = (0.0, 0.0, 1.0, 0.0, 1.0)


def _loss(s):
    return float(np.sum(s.density * s.cell_size * (s.x_Cp + s.x_CO)))


def test_config4_adjoint_fifty_draws():
    from prism3d_gb300 import fields
    from prism3d_gb300.adjoint import SteadyProblem
    dens, g0, nside, zeta, cell = fields.workload("cube32", seed=1)
    box = cell * dens.shape[0]
    kw = dict(zeta_CR_0=zeta, nside_rt=nside, tol=1e-11, n_allow=8, max_iterations=20000)
    P0 = SteadyProblem(dens, box, g0, **kw)
    T = P0.solve(np.zeros(9)).T_gas.copy()
    P0.close()
    P = SteadyProblem(dens, box, g0, T_fixed=T, w_columns=W, w_T=0.0, **kw)
    s = P.solve(np.zeros(9))
    r = s.adjoint(w_columns=W, w_T=0.0, density_gradient=True)
    assert r["converged"], r["message"]
    grad, grad_n = r["grad"].copy(), r["grad_ln_nH"].copy()
    adj, fd = [], []
    for j in range(9):
        e = np.zeros(9)
        e[j] = H
        vals = [_loss(P.solve(sg * e)) for sg in (1, -1)]
        adj.append(grad[j])
        fd.append((vals[0] - vals[1]) / (2 * H))
    P.close()
    rng = np.random.default_rng(40)
    cells = set()
    while len(cells) < 41:
        cells.add(tuple(int(v) for v in rng.integers(0, dens.shape[0], 3)))
    for c in sorted(cells):
        vals = []
        for sg in (1, -1):
            D = dens.copy()
            D[c] *= np.exp(sg * H)
            Q = SteadyProblem(D, box, g0, T_fixed=T, w_columns=W, w_T=0.0, **kw)
            vals.append(_loss(Q.solve(np.zeros(9))))
            Q.close()
        adj.append(grad_n[c])
        fd.append((vals[0] - vals[1]) / (2 * H))
    adj, fd = np.array(adj), np.array(fd)
    scale = np.max(np.abs(fd))
    assert scale > 0
    err = np.abs(adj - fd)
    assert err.max() <= 1e-4 * scale, (err.max() / scale, int(np.argmax(err)))
    big = np.abs(fd) > 1e-2 * scale
    assert np.all(err[big] <= 1e-3 * np.abs(fd[big])), np.max(err[big] / np.abs(fd[big]))
