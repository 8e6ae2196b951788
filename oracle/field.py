"""FP64 numpy restatement of HyMD's particle-field path (test infrastructure only).

Follows, step by step and in real space where the reference works in real
space:
  update_field                hymd/field.py:428-616
  compute_field_force         hymd/field.py:152-200
  compute_field_and_kinetic_energy  hymd/field.py:619-703
  compute_self_energy_q       hymd/field.py:203-238
  update_field_force_q        hymd/field.py:241-403 (PIC_Spectral)
  update_field_force_q_GPE    hymd/field.py:764-1112 (PIC_Spectral_GPE, with the
                              energy of compute_field_energy_q_GPE :706-761)
  comp_laplacian              hymd/field.py:406-425
  comp_pressure               hymd/pressure.py:9-179

Conventions of the mesh library the reference calls (pmesh, third-party and
not vendored with HyMD), restated here:
  * CIC window with mesh nodes at x = i*h, h = L/n; a particle at grid
    coordinate s = x/h deposits (1-|s-i|) per axis onto nodes floor(s) and
    floor(s)+1, periodic.  Readout uses the same weights.
  * r2c is normalised by 1/M (M = number of mesh points); c2r is unnormalised,
    so c2r(r2c(f)) == f.
  * Wavevectors k_d = 2 pi m / L_d, m in fftfreq order on the full axes and
    0..n/2 on the last (half) axis.  The filter uses |k|^2 including the
    Nyquist modes.  For the spectral gradient -i k_d, the Nyquist index of
    axis d contributes zero (the odd derivative of a real field has no
    real-valued Nyquist component); the Gaussian filter makes the difference
    with other conventions at most exp(-sigma^2 k_N^2) of the signal.
  * k.normp(p=2, zeromode=1) is sum_d k_d^2 with the k=0 entry replaced by 1.
"""
import numpy as np

from .hamiltonian import filter_H

COULOMB_CONSTANT = 138.935458  # kJ nm mol^-1 e^-2, hymd/input_parser.py:160


def _mesh(n):
    n = np.asarray(n, dtype=np.int64).reshape(-1)
    if n.size == 1:
        n = np.repeat(n, 3)
    return tuple(int(x) for x in n)


def kvectors(n, box):
    """k_x (n0,1,1), k_y (1,n1,1), k_z (1,1,n2//2+1) for the r2c layout."""
    n = _mesh(n)
    box = np.asarray(box, dtype=np.float64)
    kx = 2 * np.pi / box[0] * np.fft.fftfreq(n[0], 1.0 / n[0])
    ky = 2 * np.pi / box[1] * np.fft.fftfreq(n[1], 1.0 / n[1])
    kz = 2 * np.pi / box[2] * np.arange(n[2] // 2 + 1)
    return kx[:, None, None], ky[None, :, None], kz[None, None, :]


def kvectors_gradient(n, box):
    """Same as kvectors but with the Nyquist index of each axis set to zero."""
    n = _mesh(n)
    kx, ky, kz = (k.copy() for k in kvectors(n, box))
    if n[0] % 2 == 0:
        kx[n[0] // 2, 0, 0] = 0.0
    if n[1] % 2 == 0:
        ky[0, n[1] // 2, 0] = 0.0
    if n[2] % 2 == 0:
        kz[0, 0, n[2] // 2] = 0.0
    return kx, ky, kz


def k2(n, box):
    kx, ky, kz = kvectors(n, box)
    return kx * kx + ky * ky + kz * kz


# Threads for the transforms (scipy.fft when present); the timed CPU baseline
# sets this to the host core count.
FFT_WORKERS = 1


def r2c(grid):
    try:
        import scipy.fft as sf
        return sf.rfftn(grid, workers=FFT_WORKERS) / grid.size
    except ImportError:
        return np.fft.rfftn(grid) / grid.size


def c2r(spec, n):
    n = _mesh(n)
    M = n[0] * n[1] * n[2]
    try:
        import scipy.fft as sf
        return sf.irfftn(spec * M, s=n, axes=(0, 1, 2), workers=FFT_WORKERS)
    except ImportError:
        return np.fft.irfftn(spec * M, s=n, axes=(0, 1, 2))


def _cic_weights(pos, n, box):
    n = np.asarray(_mesh(n))
    box = np.asarray(box, dtype=np.float64)
    s = np.asarray(pos, dtype=np.float64) * (n / box)[None, :]
    i0 = np.floor(s).astype(np.int64)
    f = s - i0
    return i0, f, n


def cic_paint(pos, weight, n, box):
    """Sum_i weight_i W_CIC(g - r_i) on an (n0,n1,n2) grid (pmesh paint)."""
    i0, f, nn = _cic_weights(pos, n, box)
    weight = np.broadcast_to(np.asarray(weight, dtype=np.float64), (len(i0),))
    grid = np.zeros(int(np.prod(nn)), dtype=np.float64)
    for dx in (0, 1):
        wx = f[:, 0] if dx else 1.0 - f[:, 0]
        ix = (i0[:, 0] + dx) % nn[0]
        for dy in (0, 1):
            wy = f[:, 1] if dy else 1.0 - f[:, 1]
            iy = (i0[:, 1] + dy) % nn[1]
            for dz in (0, 1):
                wz = f[:, 2] if dz else 1.0 - f[:, 2]
                iz = (i0[:, 2] + dz) % nn[2]
                flat = (ix * nn[1] + iy) * nn[2] + iz
                grid += np.bincount(flat, weights=weight * wx * wy * wz, minlength=grid.size)
    return grid.reshape(tuple(nn))


def cic_readout(grid, pos, n, box):
    """Sum over the 8 CIC corners of W_CIC * grid (pmesh readout)."""
    i0, f, nn = _cic_weights(pos, n, box)
    out = np.zeros(len(i0), dtype=np.float64)
    for dx in (0, 1):
        wx = f[:, 0] if dx else 1.0 - f[:, 0]
        ix = (i0[:, 0] + dx) % nn[0]
        for dy in (0, 1):
            wy = f[:, 1] if dy else 1.0 - f[:, 1]
            iy = (i0[:, 1] + dy) % nn[1]
            for dz in (0, 1):
                wz = f[:, 2] if dz else 1.0 - f[:, 2]
                iz = (i0[:, 2] + dz) % nn[2]
                out += wx * wy * wz * grid[ix, iy, iz]
    return out


def update_field(positions, types, n_types, mesh, box, masses, functional, sigma,
                 compute_potential=False):
    """hymd/field.py:428-616 in FP64.

    Returns dict with phi (filtered densities, real), phi_fourier (H * r2c(phi)),
    force_mesh [t][d] (real) and, when requested, v_ext [t] (real).
    """
    n = _mesh(mesh)
    box = np.asarray(box, dtype=np.float64)
    V = float(np.prod(box))
    dV = V / (n[0] * n[1] * n[2])
    K2 = k2(n, box)
    H = filter_H(K2, sigma)
    kg = kvectors_gradient(n, box)
    phi, phi_fourier = [], []
    for t in range(n_types):
        sel = types == t
        g = cic_paint(positions[sel], masses[t], n, box) / dV
        spec = r2c(g) * H
        phi_fourier.append(spec)
        phi.append(c2r(spec, n))
    force_mesh, v_ext = [], []
    for t in range(n_types):
        v = functional.v_ext(t, phi)
        vk = r2c(v) * H
        force_mesh.append([c2r(-1j * kg[d] * vk, n) for d in range(3)])
        if compute_potential:
            v_ext.append(c2r(vk, n))
    return dict(phi=phi, phi_fourier=phi_fourier, force_mesh=force_mesh, v_ext=v_ext)


def compute_field_force(force_mesh, positions, types, n_types, mesh, box):
    """hymd/field.py:197-200: force[types==t, d] = readout(force_mesh[t][d])."""
    F = np.zeros((len(positions), 3), dtype=np.float64)
    for t in range(n_types):
        sel = types == t
        for d in range(3):
            F[sel, d] = cic_readout(force_mesh[t][d], positions[sel], mesh, box)
    return F


def field_energy(phi, functional, mesh, box):
    """W = sum_g w_0(phi~) dV (hymd/field.py:688-693)."""
    n = _mesh(mesh)
    dV = float(np.prod(box)) / (n[0] * n[1] * n[2])
    return float(np.sum(functional.w(phi) * dV))


def kinetic_energy(velocities, mass):
    """hymd/field.py:695."""
    return float(0.5 * mass * np.sum(np.asarray(velocities, dtype=np.float64) ** 2))


def self_energy_q(charges, sigma, dielectric_const):
    """hymd/field.py:203-238."""
    pref = COULOMB_CONSTANT / dielectric_const * np.sqrt(1.0 / (2.0 * np.pi * sigma * sigma))
    return float(pref * np.sum(np.asarray(charges, dtype=np.float64) ** 2))


def update_field_force_q(charges, positions, mesh, box, sigma, dielectric_const):
    """hymd/field.py:356-403 (PIC_Spectral).  Returns phi_q, psi, elec_field, forces."""
    n = _mesh(mesh)
    box = np.asarray(box, dtype=np.float64)
    dV = float(np.prod(box)) / (n[0] * n[1] * n[2])
    fac = COULOMB_CONSTANT / dielectric_const
    phi_q = cic_paint(positions, charges, n, box) / dV
    K2 = k2(n, box)
    spec = r2c(phi_q) * filter_H(K2, sigma)
    knorm = K2.copy()
    knorm[0, 0, 0] = 1.0
    psi_k = 4.0 * np.pi * fac * spec / knorm
    psi = c2r(psi_k, n)
    kg = kvectors_gradient(n, box)
    elec_field = [c2r(-1j * kg[d] * psi_k, n) for d in range(3)]
    forces = np.stack(
        [np.asarray(charges, dtype=np.float64) * cic_readout(elec_field[d], positions, n, box)
         for d in range(3)], axis=1)
    return dict(phi_q=phi_q, psi=psi, elec_field=elec_field, forces=forces, psi_fourier=psi_k)


def field_q_energy(phi_q, psi, self_energy, mesh, box):
    """W_elec = sum_g (1/2 phi_q psi - E_self / V) dV (hamiltonian w_elec, field.py:698-699)."""
    n = _mesh(mesh)
    V = float(np.prod(box))
    dV = V / (n[0] * n[1] * n[2])
    return float(np.sum((0.5 * phi_q * psi - self_energy / V) * dV))


def comp_laplacian(phi_fourier, mesh, box):
    """hymd/field.py:406-425: lap[t][d] = c2r(-k_d^2 phi_fourier[t])."""
    n = _mesh(mesh)
    k = kvectors(n, box)
    return [[c2r(-(k[d] ** 2) * pf, n) for d in range(3)] for pf in phi_fourier]


def comp_pressure(phi, phi_fourier, functional, velocities, mass, mesh, box, sigma,
                  bond_pr, angle_pr, phi_q=None, psi=None, self_energy=0.0,
                  type_charges=None):
    """hymd/pressure.py:9-179 in FP64; returns the (18,) vector."""
    n = _mesh(mesh)
    box = np.asarray(box, dtype=np.float64)
    V = float(np.prod(box))
    dV = V / (n[0] * n[1] * n[2])
    T = len(phi)
    w = functional.w(phi) * dV
    if psi is not None:
        w = w + (0.5 * phi_q * psi - self_energy / V) * dV
    p_kin = 2.0 / (3.0 * V) * kinetic_energy(velocities, mass)
    p0 = -1.0 / V * np.sum(w)
    V_bar = [functional.V_bar_0(t, phi) + (type_charges[t] * psi if psi is not None else 0.0)
             for t in range(T)]
    p1 = sum(np.sum(dV / V * V_bar[t] * phi[t]) for t in range(T))
    lap = comp_laplacian(phi_fourier, n, box)
    p2 = np.array([sum(np.sum(dV / V * sigma ** 2 * V_bar[t] * lap[t][d]) for t in range(T))
                   for d in range(3)])
    p_bond = np.asarray(bond_pr, dtype=np.float64) / V
    p_angle = np.asarray(angle_pr, dtype=np.float64) / V
    p_dih = np.zeros(3)
    p_tot = p_kin + p0 + p1 + p2 + p_bond + p_angle + p_dih
    return np.array([p_kin, p0, p1, *p2, *p_bond, *p_angle, *p_dih, *p_tot])


def gaussian_core_energy(r, kappa, sigma, rho0, names=None, chi=None, a_shift=True):
    """Continuum energy of Gaussian-filtered point particles with a quadratic
    functional (the analytic known answer of test/test_hamiltonian.py:165-360):
    E = N/c + sum_{i<j} 2 exp(-r_ij^2/(4 sigma^2))/c  [- N/(2 kappa) with the
    '-a' shift], c = 16 pi^{3/2} kappa sigma^3 rho0, plus for chi pairs
    sum 2 kappa chi_ij exp(-r_ij^2/(4 sigma^2))/c."""
    r = np.asarray(r, dtype=np.float64)
    N = len(r)
    pi32 = np.arccos(-1.0) ** 1.5
    c = 16.0 * pi32 * kappa * sigma ** 3 * rho0
    E = N / c
    for i in range(N):
        for j in range(i + 1, N):
            d = r[i] - r[j]
            E += 2 * np.exp(-np.dot(d, d) / (4.0 * sigma ** 2)) / c
    if a_shift:
        E -= 0.5 * N / kappa
    if chi is not None:
        for i in range(N):
            for j in range(i + 1, N):
                if names[i] != names[j]:
                    d = r[i] - r[j]
                    E += 2 * kappa * chi[tuple(sorted((names[i], names[j])))] / c * np.exp(
                        -np.dot(d, d) / (4.0 * sigma ** 2))
    return E


def _conv(diff, kind):
    """Convergence measures of hymd/main.py:141-165 over the mesh: max_diff
    (the default), csum (sum), euclidean_norm (pmesh cnorm: sum of squares)."""
    if kind == "csum":
        return float(np.sum(diff))
    if kind == "euclidean_norm":
        return float(np.sum(diff * diff))
    return float(np.max(diff))


def gpe_step(phi_tilde, charges, positions, types, n_types, mesh, box, sigma, eps_type,
             type_charges, state, conv_crit=1e-6, mixing=0.6, conv_kind="max_diff",
             max_iter=100, coulomb_constant=COULOMB_CONSTANT):
    """PIC_Spectral_GPE electrostatics (hymd/field.py:764-1112) and its energy
    (:706-761) in FP64.

    phi_tilde: list of the filtered type densities (what update_field leaves
    in phi).  state: dict of the grids the reference keeps between calls --
    phi_eps, pol_prev, contrib (its masked divisions leave old values where
    the mask is false) -- phi_eps and contrib are updated in place; pol_prev
    is the starting polarisation and is not written, because the reference
    rebinds phi_pol_prev and phi_pol locally (field.py:1010-1024) and its
    caller's grids never change.  Returns dict(forces, psi, elec_field,
    phi_eps, elec_dot, Vbar, energy, iterations)."""
    n = _mesh(mesh)
    box = np.asarray(box, dtype=np.float64)
    M = n[0] * n[1] * n[2]
    dV = float(np.prod(box)) / M
    K2 = k2(n, box)
    H = filter_H(K2, sigma)
    kg = kvectors_gradient(n, box)
    knorm = K2.copy()
    knorm[0, 0, 0] = 1.0
    pos = np.asarray(positions, dtype=np.float64)
    rho = cic_paint(pos, np.asarray(charges, np.float64), n, box) / dV
    rho_t = c2r(r2c(rho) * H, n)
    tot = np.zeros(n)
    num = np.zeros(n)
    for t in range(n_types):
        tot += phi_tilde[t]
        num += eps_type[t] * phi_tilde[t]
    m_tot = tot > 1e-6
    phi_eps = state["phi_eps"]
    phi_eps[m_tot] = num[m_tot] / tot[m_tot]
    eps_k = r2c(phi_eps)
    m_eps = phi_eps > 1e-6
    q = rho_t.copy()
    q[m_eps] = rho_t[m_eps] / phi_eps[m_eps]
    eta = []
    for d in range(3):
        g = c2r(1j * kg[d] * eps_k, n)
        g[m_eps] = g[m_eps] / phi_eps[m_eps]
        eta.append(g)
    pol_prev = state["pol_prev"].copy()
    it, delta = 0, 1.0
    while it < max_iter and delta > conv_crit:
        X = r2c(q + pol_prev)
        E = [c2r(X * (-1j * kg[d]) / knorm, n) for d in range(3)]
        pol = -(eta[0] * E[0] + eta[1] * E[1] + eta[2] * E[2])
        pol = mixing * pol + (1.0 - mixing) * pol_prev
        delta = _conv(np.abs(pol - pol_prev), conv_kind)
        pol_prev = pol.copy()
        it += 1
    eps0_inv = coulomb_constant * 4.0 * np.pi
    psik = r2c(eps0_inv * (q + pol_prev)) / knorm
    psi = c2r(psik, n)
    E = [c2r(-1j * kg[d] * psik, n) for d in range(3)]
    dot = E[0] * E[0] + E[1] * E[1] + E[2] * E[2]
    contrib = state["contrib"]
    contrib[m_tot] = dot[m_tot] / tot[m_tot]
    Vbar = [type_charges[t] * psi - (0.5 / eps0_inv) * (eps_type[t] - phi_eps) * contrib
            for t in range(n_types)]
    F = np.zeros((len(pos), 3))
    for t in range(n_types):
        sel = types == t
        Vk = r2c(Vbar[t]) * H
        for d in range(3):
            F[sel, d] = cic_readout(c2r(-1j * kg[d] * Vk, n), pos[sel], n, box)
    energy = dV * 0.5 / eps0_inv * float(np.sum(phi_eps * dot))
    return dict(forces=F, psi=psi, elec_field=E, phi_eps=phi_eps.copy(), elec_dot=dot,
                Vbar=Vbar, energy=energy, iterations=it)
