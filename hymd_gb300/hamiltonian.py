"""Interaction energy functionals -- the plugin boundary of the field path.

Mirrors hymd/hamiltonian.py (Hamiltonian :16-71, SquaredPhi :74-204,
DefaultNoChi :207-319, DefaultWithChi :322-486, get_hamiltonian :489-512):
same class names, constructor arguments and attributes (H, w, w_0, v_ext[t],
V_bar_0[t], V_bar[t], w_elec).  The pointwise callables work elementwise on
numpy arrays or torch tensors.

The GPU force path needs the functional in closed form: every reference
functional is quadratic in the filtered densities,
    w(phi) = 1/2 phi.Q.phi + b.phi + c,
and `quadratic_form(h)` returns (Q, b, c, sigma).  A user subclass that
overrides `w_0` with a non-quadratic functional, or replaces the filter `H`,
raises NotImplementedError there: there is no CPU fallback.
"""
import numpy as np


class Hamiltonian:
    """Superclass: filter H(k, v) = v exp(-sigma^2 |k|^2 / 2) and rho0 / a
    defaults (hymd/hamiltonian.py:34-71)."""

    gaussian_filter = True

    def __init__(self, config):
        self.config = config
        self._setup()

    def _setup(self):
        c = self.config
        if getattr(c, "simulation_volume", None) is None:
            c.simulation_volume = float(np.prod(np.asarray(c.box_size, dtype=np.float64)))
        if not c.barostat:
            c.rho0 = c.n_particles / c.simulation_volume
            c.a = c.rho0
        if not c.rho0:
            c.rho0 = c.n_particles / c.simulation_volume
        if not c.self_energy:
            c.self_energy = 0.0
        sigma = c.sigma

        def H(k, v):
            k = np.asarray(k)
            return v * np.exp(-0.5 * sigma ** 2 * (k[0] ** 2 + k[1] ** 2 + k[2] ** 2))

        self.H = H
        self._H_default = H

    # ------------------------------------------------------------------
    def _install(self, Q, b, c):
        self.Q = np.asarray(Q, dtype=np.float64)
        self.b = np.asarray(b, dtype=np.float64)
        self.c = float(c)
        T = self.Q.shape[0]
        Q_, b_, c_ = self.Q, self.b, self.c
        cfg = self.config

        def w(phi):
            out = c_ + 0.0 * phi[0]
            for i in range(T):
                out = out + b_[i] * phi[i]
                for j in range(T):
                    out = out + 0.5 * Q_[i, j] * phi[i] * phi[j]
            return out

        def make_v(t):
            def v(phi):
                out = b_[t] + 0.0 * phi[0]
                for j in range(T):
                    out = out + Q_[t, j] * phi[j]
                return out
            return v

        def w_elec(args, volume=cfg.simulation_volume, self_energy=cfg.self_energy):
            phi_q, psi = args
            return 0.5 * phi_q * psi - self_energy / volume

        charges = cfg.type_charges if cfg.type_charges is not None else [0.0] * T

        def make_vbar(t):
            v0 = make_v(t)

            def vb(args):
                phi, psi = args
                return v0(phi) + charges[t] * psi
            return vb

        self.w_0 = w
        self.v_ext = [make_v(t) for t in range(T)]
        self.V_bar_0 = [make_v(t) for t in range(T)]
        self.V_bar = [make_vbar(t) for t in range(T)]
        self.w_elec = w_elec
        if cfg.coulombtype == "PIC_Spectral":
            def w_full(args):
                phi, phi_q, psi = args
                return w(phi) + w_elec((phi_q, psi))
            self.w = w_full
        else:
            self.w = w


class SquaredPhi(Hamiltonian):
    """w = 1/(2 kappa rho0) (sum_t phi_t)^2 (hymd/hamiltonian.py:74-204)."""

    def __init__(self, config):
        super().__init__(config)
        c = self.config
        T = c.n_types
        inv = 1.0 / (c.kappa * c.rho0)
        self._install(np.full((T, T), inv), np.zeros(T), 0.0)


class DefaultNoChi(Hamiltonian):
    """w = 1/(2 kappa rho0) (sum_t phi_t - a)^2 (hymd/hamiltonian.py:207-319)."""

    def __init__(self, config):
        super().__init__(config)
        c = self.config
        T = c.n_types
        inv = 1.0 / (c.kappa * c.rho0)
        self._install(np.full((T, T), inv), np.full(T, -c.a * inv), 0.5 * c.a * c.a * inv)


class DefaultWithChi(Hamiltonian):
    """w = sum_{i<j} chi_ij phi_i phi_j / rho0 + 1/(2 kappa rho0) (sum phi - a)^2
    (hymd/hamiltonian.py:322-486).  chi_ii is ignored, as in the reference."""

    def __init__(self, config, unique_names, type_to_name_map):
        super().__init__(config)
        c = self.config
        self.type_to_name_map = type_to_name_map
        self.chi_type_dictionary = {
            tuple(sorted([x.atom_1, x.atom_2])): x.interaction_energy for x in c.chi}
        T = c.n_types
        inv = 1.0 / (c.kappa * c.rho0)
        Q = np.full((T, T), inv)
        for i in range(T):
            for j in range(T):
                if i != j:
                    key = tuple(sorted([type_to_name_map[i], type_to_name_map[j]]))
                    Q[i, j] += self.chi_type_dictionary.get(key, 0.0) / c.rho0
        self._install(Q, np.full(T, -c.a * inv), 0.5 * c.a * c.a * inv)


def get_hamiltonian(config):
    """hymd/hamiltonian.py:489-512."""
    name = config.hamiltonian.lower()
    if name == "defaultnochi":
        return DefaultNoChi(config)
    if name == "defaultwithchi":
        return DefaultWithChi(config, config.unique_names, config.type_to_name_map)
    if name == "squaredphi":
        return SquaredPhi(config)
    raise ValueError(f"unknown hamiltonian {config.hamiltonian!r}")


def quadratic_form(h, n_types=None):
    """(Q, b, c, sigma) of a Hamiltonian-like object.

    Objects of this module carry Q/b/c directly.  For any other object with a
    `w_0(phi_list)` callable (e.g. a user subclass written against the
    reference API) the coefficients are recovered by evaluating w_0 at
    0, e_i, 2 e_i and e_i + e_j, and then checked on random points; a
    functional that is not quadratic raises NotImplementedError.
    """
    cached = getattr(h, "_hpf_quadratic", None)
    if cached is not None:
        return cached
    cfg = h.config
    sigma = float(cfg.sigma)
    if getattr(h, "H", None) is not None and getattr(h, "_H_default", None) is not None:
        if h.H is not h._H_default:
            raise NotImplementedError("a replaced filter H has no GPU implementation")
    if hasattr(h, "Q") and hasattr(h, "b") and hasattr(h, "c"):
        out = (np.asarray(h.Q, np.float64), np.asarray(h.b, np.float64), float(h.c), sigma)
    else:
        T = n_types if n_types is not None else cfg.n_types

        def w(vec):
            return float(np.asarray(h.w_0([np.array([x], dtype=np.float64) for x in vec])).reshape(-1)[0])

        z = np.zeros(T)
        c = w(z)
        we = np.array([w(np.eye(T)[i]) for i in range(T)])
        w2 = np.array([w(2 * np.eye(T)[i]) for i in range(T)])
        Q = np.zeros((T, T))
        for i in range(T):
            Q[i, i] = w2[i] - 2 * we[i] + c
            for j in range(i + 1, T):
                Q[i, j] = Q[j, i] = w(np.eye(T)[i] + np.eye(T)[j]) - we[i] - we[j] + c
        b = we - c - 0.5 * np.diag(Q)
        rng = np.random.default_rng(0)
        for _ in range(4):
            x = rng.uniform(0.0, 3.0, T)
            ref = w(x)
            val = 0.5 * x @ Q @ x + b @ x + c
            if not np.isclose(ref, val, rtol=1e-9, atol=1e-9 * (1 + abs(ref))):
                raise NotImplementedError(
                    "interaction functional is not quadratic in phi; the GPU field path "
                    "supports quadratic functionals only")
        out = (Q, b, c, sigma)
    try:
        h._hpf_quadratic = out
    except AttributeError:
        pass
    return out
