"""Adjoint of the field energy (hymd_gb300.adjoint) against FP64 central
finite differences of the oracle energy.

Tolerances: parameter gradients (chi, kappa, sigma) within 1e-5 relative of
the FP64 finite difference; position gradients within 1e-4 relative RMS
(FP32 potential grids and readout); W itself within 1e-7 relative.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import field as of  # noqa: E402
from oracle import hamiltonian as oh  # noqa: E402

PARAM_RTOL = 1e-5
POS_RTOL = 1e-4


def _system(seed=3, n=3000, T=3, mesh=(24, 24, 24), box=(5.0, 5.5, 6.0)):
    rng = np.random.default_rng(seed)
    box = np.asarray(box, np.float64)
    r = (rng.uniform(0, 1, (n, 3)) * box).astype(np.float32)
    r[: n // 2] = np.mod(box / 2 + rng.normal(0, 0.7, (n // 2, 3)), box).astype(np.float32)
    types = rng.integers(0, T, n).astype(np.int32)
    chi = np.zeros((T, T))
    for i in range(T):
        for j in range(i + 1, T):
            chi[i, j] = chi[j, i] = rng.uniform(5, 30)
    masses = list(rng.uniform(0.8, 1.2, T))
    rho0 = n / float(np.prod(box))
    return r, types, chi, masses, rho0, mesh, box


def _w_oracle(r, types, T, mesh, box, m, kind, chi, kappa, sigma, rho0, a):
    fun = oh.quadratic_from_params(kind, T, kappa, rho0, a, chi)
    ref = of.update_field(np.asarray(r, np.float64), types, T, mesh, box, m, fun, sigma)
    return of.field_energy(ref["phi"], fun, mesh, box)


@pytest.mark.parametrize("kind", ["DefaultWithChi", "DefaultNoChi", "SquaredPhi"])
def test_parameter_gradients_match_finite_differences(kind):
    from hymd_gb300.adjoint import field_energy
    from hymd_gb300.field import ParticleMesh
    r, types, chi, m, rho0, mesh, box = _system()
    T = chi.shape[0]
    kappa, sigma, a = 0.05, 0.5, rho0 * 1.02
    pm = ParticleMesh(mesh, box, T)
    R = torch.as_tensor(r, device="cuda")
    Ty = torch.as_tensor(types, device="cuda")
    chi_t = torch.tensor(chi, dtype=torch.float64, requires_grad=True)
    k_t = torch.tensor(kappa, dtype=torch.float64, requires_grad=True)
    s_t = torch.tensor(sigma, dtype=torch.float64, requires_grad=True)
    W = field_energy(R, Ty, pm, m, chi_t, k_t, s_t, rho0, a, kind=kind)
    W.backward()
    args = (r, types, T, mesh, box, m, kind)
    W0 = _w_oracle(*args, chi, kappa, sigma, rho0, a)
    assert float(W.detach()) == pytest.approx(W0, rel=1e-7)
    # sigma and kappa: central differences in FP64
    for name, grad, x0, h in (("sigma", s_t.grad, sigma, 1e-5), ("kappa", k_t.grad, kappa, 1e-7)):
        def w_at(x):
            kk, ss = (kappa, x) if name == "sigma" else (x, sigma)
            return _w_oracle(*args, chi, kk, ss, rho0, a)
        fd = (w_at(x0 + h) - w_at(x0 - h)) / (2 * h)
        assert float(grad) == pytest.approx(fd, rel=PARAM_RTOL), name
    G = chi_t.grad.numpy()
    assert np.allclose(G, G.T) and np.all(np.diag(G) == 0)
    if kind == "DefaultWithChi":
        h = 1e-4
        for i, j in ((0, 1), (0, 2), (1, 2)):
            cp, cm = chi.copy(), chi.copy()
            cp[i, j] += h
            cp[j, i] += h
            cm[i, j] -= h
            cm[j, i] -= h
            fd = (_w_oracle(*args, cp, kappa, sigma, rho0, a)
                  - _w_oracle(*args, cm, kappa, sigma, rho0, a)) / (2 * h)
            # one pair moved in both entries: dW = (G_ij + G_ji) d
            assert G[i, j] + G[j, i] == pytest.approx(fd, rel=PARAM_RTOL), (i, j)
    else:
        assert np.all(G == 0)
    pm.check_errors()


def test_position_gradient_matches_finite_differences_and_force():
    from hymd_gb300.adjoint import field_energy
    from hymd_gb300.field import ParticleMesh
    r, types, chi, m, rho0, mesh, box = _system(seed=4)
    T = chi.shape[0]
    kappa, sigma, a = 0.05, 0.5, rho0
    pm = ParticleMesh(mesh, box, T)
    R = torch.as_tensor(r, device="cuda").requires_grad_(True)
    Ty = torch.as_tensor(types, device="cuda")
    W = field_energy(R, Ty, pm, m, chi, kappa, sigma, rho0, a)
    W.backward()
    g = R.grad.cpu().numpy().astype(np.float64)
    args = (types, T, mesh, box, m, "DefaultWithChi", chi, kappa, sigma, rho0, a)
    rng = np.random.default_rng(0)
    h_mesh = np.asarray(box) / np.asarray(mesh)
    eps = 1e-3
    got, want = [], []
    for i in rng.choice(len(r), 24, replace=False):
        for d in range(3):
            # skip windows that cross a cell boundary (W is piecewise quadratic)
            f = (float(r[i, d]) / h_mesh[d]) % 1.0
            if min(f, 1.0 - f) * h_mesh[d] < 2 * eps:
                continue
            rp = r.astype(np.float64)
            rm = rp.copy()
            rp[i, d] += eps
            rm[i, d] -= eps
            fd = (_w_oracle(rp, *args) - _w_oracle(rm, *args)) / (2 * eps)
            got.append(g[i, d])
            want.append(fd)
    got, want = np.array(got), np.array(want)
    assert len(got) >= 40
    assert np.sqrt(np.mean((got - want) ** 2)) <= POS_RTOL * np.sqrt(np.mean(want ** 2))
    # the spectral-readout force agrees with -dW/dx up to the O(h^2) gap
    fun = oh.quadratic_from_params("DefaultWithChi", T, kappa, rho0, a, chi)
    ref = of.update_field(r.astype(np.float64), types, T, mesh, box, m, fun, sigma)
    F = of.compute_field_force(ref["force_mesh"], r.astype(np.float64), types, T, mesh, box)
    cos = np.sum(-g * F) / (np.linalg.norm(g) * np.linalg.norm(F))
    assert cos > 0.9
    pm.check_errors()


def test_chi_fit_to_target_energy_in_one_newton_step():
    """W is linear in chi at fixed positions, so one Newton step along the
    adjoint gradient, d = -(W - W*) g / |g|^2, must land on a target energy W*
    made with other chi values -- a check of the gradient's direction and
    size together (the use the adjoint exists for: fitting chi)."""
    from hymd_gb300.adjoint import field_energy
    from hymd_gb300.field import ParticleMesh
    r, types, chi, m, rho0, mesh, box = _system(seed=5)
    T = chi.shape[0]
    pm = ParticleMesh(mesh, box, T)
    R = torch.as_tensor(r, device="cuda")
    Ty = torch.as_tensor(types, device="cuda")
    target = float(field_energy(R, Ty, pm, m, chi, 0.05, 0.5, rho0, rho0))
    c = torch.tensor(chi + 3.0 * (1 - np.eye(T)), dtype=torch.float64, requires_grad=True)
    W = field_energy(R, Ty, pm, m, c, 0.05, 0.5, rho0, rho0)
    W.backward()
    g = c.grad
    w1 = float(W.detach())
    with torch.no_grad():
        c2 = c - (w1 - target) * g / (g * g).sum()
    W2 = float(field_energy(R, Ty, pm, m, c2, 0.05, 0.5, rho0, rho0))
    assert abs(W2 - target) <= 1e-6 * abs(w1 - target)
