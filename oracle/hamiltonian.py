"""Oracle restatement of HyMD's interaction functionals (test infrastructure only).

Follows hymd/hamiltonian.py:
  Hamiltonian._setup  :34-71   rho0 = N/V (and a = rho0) without a barostat; H filter
  SquaredPhi          :74-204  w = 1/(2 kappa rho0) (sum phi)^2
  DefaultNoChi        :207-319 w = 1/(2 kappa rho0) (sum phi - a)^2
  DefaultWithChi      :322-486 w = sum_{i<j} chi_ij phi_i phi_j / rho0
                                   + 1/(2 kappa rho0) (sum phi - a)^2
All three are quadratic in the filtered densities, so each is represented as
    w(phi) = 1/2 phi^T Q phi + b^T phi + c,   v_ext[t] = dw/dphi_t = (Q phi)_t + b_t.
The diagonal chi_ii is ignored, as in the reference (hamiltonian.py:393-412).
"""
import numpy as np


class QuadraticFunctional:
    def __init__(self, Q, b, c):
        self.Q = np.asarray(Q, dtype=np.float64)
        self.b = np.asarray(b, dtype=np.float64)
        self.c = float(c)
        self.n_types = self.Q.shape[0]

    def w(self, phi):
        """Pointwise energy density on a list of grids (hamiltonian.py:475)."""
        T = self.n_types
        out = np.full(np.shape(phi[0]), self.c, dtype=np.float64)
        for i in range(T):
            out += self.b[i] * phi[i]
            for j in range(T):
                out += 0.5 * self.Q[i, j] * phi[i] * phi[j]
        return out

    def v_ext(self, t, phi):
        """dw/dphi_t on grids (hamiltonian.py:470-473)."""
        out = np.full(np.shape(phi[0]), self.b[t], dtype=np.float64)
        for j in range(self.n_types):
            out += self.Q[t, j] * phi[j]
        return out

    V_bar_0 = v_ext


def quadratic_from_params(kind, n_types, kappa, rho0, a=None, chi=None):
    """Q, b, c of the three reference functionals.

    chi: (T,T) symmetric matrix of chi_ij (diagonal ignored) for DefaultWithChi.
    """
    kind = kind.lower()
    inv = 1.0 / (kappa * rho0)
    Q = np.full((n_types, n_types), inv)
    b = np.zeros(n_types)
    c = 0.0
    if kind == "squaredphi":
        pass
    elif kind in ("defaultnochi", "defaultwithchi"):
        b[:] = -a * inv
        c = 0.5 * a * a * inv
        if kind == "defaultwithchi":
            chi = np.asarray(chi, dtype=np.float64)
            for i in range(n_types):
                for j in range(n_types):
                    if i != j:
                        Q[i, j] += chi[i, j] / rho0
    else:
        raise ValueError(kind)
    return QuadraticFunctional(Q, b, c)


def filter_H(k2, sigma):
    """Gaussian filter exp(-sigma^2 k^2 / 2) (hamiltonian.py:57-71)."""
    return np.exp(-0.5 * sigma * sigma * k2)


def functional_of_config(cfg):
    """The quadratic functional of a configuration's Hamiltonian
    (cfg.hamiltonian, chi list, kappa; rho0 = a = N / V unless set, as
    Hamiltonian._setup does without a barostat)."""
    T = int(cfg.n_types)
    names = list(cfg.unique_names)
    chi = np.zeros((T, T))
    for c in cfg.chi:
        i, j = names.index(c.atom_1), names.index(c.atom_2)
        chi[i, j] = chi[j, i] = c.interaction_energy
    V = float(np.prod(np.asarray(cfg.box_size, dtype=np.float64)))
    rho0 = cfg.rho0 or cfg.n_particles / V
    a = cfg.a if cfg.a is not None else rho0
    return quadratic_from_params(cfg.hamiltonian or "DefaultWithChi", T, cfg.kappa, rho0, a, chi)
