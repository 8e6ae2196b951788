"""Internal pressure -- drop-in for hymd/pressure.py:9-179 (FP64 result).

P = p_kin + p0 + p1 + p2 + p_bond + p_angle (+ p_dihedral = 0, as in the
reference) with
  p_kin = 2 KE / (3V),  p0 = -W/V,
  p1    = (dV/V) sum_t sum_g Vbar_t phi~_t,
  p2_d  = (dV/V) sigma^2 sum_t sum_g Vbar_t d_d^2 phi~_t,
  Vbar_t = v_ext_t (+ q_t psi with PIC_Spectral).
The quadratic parts are evaluated by Parseval in one k-space pass over
phi_fourier (FP64 sums), the k = 0 parts from FP64 grid means, so no
large real-space terms cancel in single precision.  phi_laplacian is
filled as in the reference (comp_laplacian) for callers that read it.
"""
import numpy as np
import torch

from . import _lib
from .field import (_pm_of, _stack_base, _sum, comp_laplacian, field_energy_parts)


def comp_pressure(phi, phi_q, psi, hamiltonian, velocities, config, phi_fourier, phi_laplacian,
                  phi_transfer, positions, bond_pr, angle_pr, comm=None):
    """Returns the (18,) float64 vector of hymd/pressure.py:155-176."""
    pm = _pm_of(phi)
    T = pm.n_types
    V = float(np.prod(pm.BoxSize))
    dV = V / pm.M
    Q, b, c, sigma = pm.set_functional(hamiltonian)
    phi_all = _stack_base(phi, (T,), torch.float32, "phi")
    phif_all = _stack_base(phi_fourier, (T,), torch.complex64, "phi_fourier")
    st = _lib.stream_ptr()
    # energy (p0) from the real-space phi~ (Parseval + exact k=0)
    W, means, _ = field_energy_parts(pm, phi_all, hamiltonian)
    # p1 / p2 quadratic parts from the filtered spectra
    sums = torch.zeros(8, dtype=torch.float64, device=pm.device)
    qt = None
    psi_k = None
    if psi is not None:
        qt = _lib.dvec(list(config.type_charges))
    _lib.call("hpf_kspace_sums", pm._h, _lib.ptr(phif_all), None, qt, _lib.ptr(sums), st)
    s = sums.cpu().numpy()
    A, Bk = s[0], s[1:4]
    vbar0 = Q @ means + b
    p1 = A + float(vbar0 @ means)
    p2 = -sigma ** 2 * Bk
    w_elec = 0.0
    if psi is not None:
        # cross terms with psi: real-space FP64 dot products (no cancellation)
        comp_laplacian(phi_fourier, phi_transfer, phi_laplacian, hamiltonian, config)
        lap_all = _stack_base(phi_laplacian, (T, 3), torch.float32, "phi_laplacian")
        for t in range(T):
            qtv = float(config.type_charges[t])
            if qtv == 0.0:
                continue
            p1 += qtv * float(_sum(pm, psi, phi_all[t])) * dV / V
            for d in range(3):
                p2[d] += sigma ** 2 * qtv * float(_sum(pm, psi, lap_all[t, d])) * dV / V
        w_elec = 0.5 * float(_sum(pm, phi_q, psi)) * dV - float(config.self_energy or 0.0)
    else:
        comp_laplacian(phi_fourier, phi_transfer, phi_laplacian, hamiltonian, config)
    vel = _lib.require_cuda(velocities, "velocities", torch.float32)
    _lib.call("hpf_sum_v2", _lib.ptr(vel), vel.shape[0], _lib.ptr(pm.ws), st)
    ke = 0.5 * float(config.mass) * float(pm.ws[0])
    p_kin = 2.0 / (3.0 * V) * ke
    p0 = -(W + w_elec) / V
    p_bond = np.asarray(_host(bond_pr), dtype=np.float64) / V
    p_angle = np.asarray(_host(angle_pr), dtype=np.float64) / V
    p_dih = np.zeros(3)
    p_tot = p_kin + p0 + p1 + p2 + p_bond + p_angle + p_dih
    return np.array([p_kin, p0, p1, *p2, *p_bond, *p_angle, *p_dih, *p_tot])


def _host(x):
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return x
