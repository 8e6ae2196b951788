"""The field oracle against the reference's own known answers:
analytic Gaussian-core energies (test/test_hamiltonian.py:165-360, 160^3, 1e-6),
CIC mass conservation (:105-128) and the reference Hamiltonian lambdas."""
import numpy as np
import pytest

from oracle import field as of
from oracle import hamiltonian as oh

R3 = np.array([[1.50, 0.75, 2.25], [2.25, 0.00, 3.00], [4.50, 1.50, 2.25]])
R5 = np.array([[1.50, 0.75, 2.25], [2.25, 0.00, 3.00], [4.50, 1.50, 2.25],
               [1.50, 1.50, 0.75], [3.00, 4.50, 1.50]])
BOX = np.array([15.0, 15.0, 15.0])


@pytest.mark.parametrize("kappa,sigma", [(0.029230985982, 0.2988365823859701),
                                         (1.299759825895, 1.2095870248085025)])
def test_gaussian_core_no_chi(kappa, sigma):
    rho0 = 3 / np.prod(BOX)
    types = np.zeros(3, int)
    for kind, shift in (("SquaredPhi", False), ("DefaultNoChi", True)):
        q = oh.quadratic_from_params(kind, 1, kappa, rho0, rho0)
        out = of.update_field(R3, types, 1, 160, BOX, [1.0], q, sigma)
        W = of.field_energy(out["phi"], q, 160, BOX)
        E = of.gaussian_core_energy(R3, kappa, sigma, rho0, a_shift=shift)
        assert W == pytest.approx(E, abs=1e-6)


@pytest.mark.parametrize("kappa,sigma", [(0.029230985982, 0.2988365823859701),
                                         (1.299759825895, 1.2095870248085025)])
def test_gaussian_core_with_chi(kappa, sigma):
    names = ["A", "A", "B", "C", "C"]
    types = np.array([0, 0, 1, 2, 2])
    rho0 = 5 / np.prod(BOX)
    chi_d = {("A", "B"): 9.6754032616815161, ("A", "C"): -13.2596290315913623,
             ("B", "C"): 0.3852001771213374}
    chi = np.zeros((3, 3))
    chi[0, 1] = chi[1, 0] = chi_d[("A", "B")]
    chi[0, 2] = chi[2, 0] = chi_d[("A", "C")]
    chi[1, 2] = chi[2, 1] = chi_d[("B", "C")]
    q = oh.quadratic_from_params("DefaultWithChi", 3, kappa, rho0, rho0, chi)
    out = of.update_field(R5, types, 3, 160, BOX, [1.0] * 3, q, sigma)
    W = of.field_energy(out["phi"], q, 160, BOX)
    E = of.gaussian_core_energy(R5, kappa, sigma, rho0, names=names, chi=chi_d)
    assert W == pytest.approx(E, abs=1e-6)


def test_cic_mass_conservation():
    r = np.array([[5.0856957005460090, 2.6917109262984917, 2.1680859811719504],
                  [0.0592355479043435, 7.4705053874595030, 0.7169198724514365],
                  [6.8662344320308580, 3.1065309079252390, 3.5621049784729850],
                  [5.5405900785250210, 6.5585020954226065, 1.3155113935992528],
                  [1.6400925628903045, 2.1325438112867725, 3.4149968975443680]])
    box = np.array([7.1598, 11.2498, 5.1009])
    types = np.array([0, 0, 1, 1, 1])
    for t, m in ((0, 2.0), (1, 3.0)):
        g = of.cic_paint(r[types == t], 1.0, 8, box)
        assert g.sum() == pytest.approx(m, abs=1e-14)
        gf = of.c2r(of.r2c(g) * oh.filter_H(of.k2(8, box), 0.2988365823859701), 8)
        assert gf.sum() == pytest.approx(m, abs=1e-13)


def test_quadratic_functionals_match_reference_lambdas(golden):
    g = golden("hamiltonian.npz")
    rho0, a, kappa, sigma = g["params"]
    ab, ac, bc = g["chi_ab_ac_bc"]
    chi = np.array([[0, ab, ac], [ab, 0, bc], [ac, bc, 0]])
    phi = [g["phi0"], g["phi1"], g["phi2"]]
    for kind in ("SquaredPhi", "DefaultNoChi", "DefaultWithChi"):
        q = oh.quadratic_from_params(kind, 3, kappa, rho0, a, chi)
        assert np.allclose(q.w(phi), g[kind + "/w0"], rtol=1e-13, atol=1e-12)
        for t in range(3):
            assert np.allclose(q.v_ext(t, phi), g[f"{kind}/v_ext{t}"], rtol=1e-13, atol=1e-12)
            assert np.allclose(q.V_bar_0(t, phi), g[f"{kind}/V_bar_0{t}"], rtol=1e-13, atol=1e-12)
        k = g[kind + "/H_k"][0]
        assert oh.filter_H(np.dot(k, k), sigma) * 0.75 == pytest.approx(g[kind + "/H_v"][0], rel=1e-14)


def test_field_force_converges_to_energy_gradient():
    """Spectral force vs central differences of W.  They differ by the
    discretisation gap (CIC-weight derivative vs spectral gradient); the gap
    must shrink when the mesh is refined at fixed sigma."""
    rng = np.random.default_rng(3)
    box = np.array([4.0, 4.0, 4.0])
    r = rng.uniform(0, 4.0, size=(40, 3))
    types = rng.integers(0, 2, 40)
    chi = np.array([[0, 20.0], [20.0, 0]])
    rho0 = 40 / 64.0
    q = oh.quadratic_from_params("DefaultWithChi", 2, 0.1, rho0, rho0, chi)
    sigma, h, i = 0.5, 1e-4, 7
    gaps = []
    for n in (16, 32):
        out = of.update_field(r, types, 2, n, box, [1.0, 1.0], q, sigma)
        F = of.compute_field_force(out["force_mesh"], r, types, 2, n, box)
        g = np.zeros(3)
        for d in range(3):
            rp = r.copy(); rp[i, d] += h
            rm = r.copy(); rm[i, d] -= h
            Wp = of.field_energy(of.update_field(rp, types, 2, n, box, [1, 1], q, sigma)["phi"], q, n, box)
            Wm = of.field_energy(of.update_field(rm, types, 2, n, box, [1, 1], q, sigma)["phi"], q, n, box)
            g[d] = (Wp - Wm) / (2 * h)
        gaps.append(np.linalg.norm(F[i] + g) / np.linalg.norm(g))
    assert gaps[1] < 0.1
    assert gaps[1] < 0.6 * gaps[0]
