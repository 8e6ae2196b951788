"""Internal pressure -- drop-in for hymd/pressure.py:9-179 (FP64 result).

P = p_kin + p0 + p1 + p2 + p_bond + p_angle (+ p_dihedral = 0, as in the
reference) with
  p_kin = 2 KE / (3V),  p0 = -(W + W_elec)/V,
  p1    = (dV/V) sum_t sum_g Vbar_t phi~_t,
  p2_d  = (dV/V) sigma^2 sum_t sum_g Vbar_t d_d^2 phi~_t,
  Vbar_t = v_ext_t (+ q_t psi with PIC_Spectral).
By Parseval, with phi~ = H phi / M and Vbar_t(k) = (Q phi~)_t + b_t delta_k0
(+ q_t psi(k)):
  p1   = A + (Q mean + b).mean [+ C0],   p2_d = -sigma^2 (B_d [+ C_d]),
where A, B, C are the FP64 half-spectrum sums of hpf_energy_fp64 computed
from the fixed-point densities of `positions` -- no large real-space terms
cancel in single precision.  phi_laplacian is filled as in the reference
(comp_laplacian) for callers that read it.
"""
import numpy as np
import torch

from . import _lib
from .field import _pm_of, comp_laplacian, energy_fp64


def comp_pressure(phi, phi_q, psi, hamiltonian, velocities, config, phi_fourier, phi_laplacian,
                  phi_transfer, positions, bond_pr, angle_pr, comm=None):
    """Returns the (18,) float64 vector of hymd/pressure.py:155-176."""
    pm = _pm_of(phi)
    # the types of the particles that update_field painted into phi
    types = getattr(pm, "last_types", None)
    if types is None:
        raise ValueError("comp_pressure needs a preceding update_field on this mesh")
    charges = None
    fac = 0.0
    qt = None
    if psi is not None:
        charges = getattr(pm, "pic_charges", None)
        fac = config.coulomb_constant / config.dielectric_const
        qt = list(config.type_charges)
    e = energy_fp64(pm, positions, types, config.m, hamiltonian, charges=charges,
                    type_charges=qt, elec_factor=fac)
    comp_laplacian(phi_fourier, phi_transfer, phi_laplacian, hamiltonian, config)
    vel = _lib.require_cuda(velocities, "velocities", torch.float32)
    _lib.call("hpf_sum_v2", _lib.ptr(vel), vel.shape[0], _lib.ptr(pm.ws), _lib.stream_ptr())
    ke = 0.5 * float(config.mass) * float(pm.ws[0])
    self_energy = float(config.self_energy or 0.0) if charges is not None else None
    return pressure_vector(e, ke, _host(bond_pr), _host(angle_pr), self_energy)


def pressure_vector(e, ke, bond_pr, angle_pr, self_energy=None):
    """The (18,) vector of hymd/pressure.py:155-176 from the FP64 sums `e`
    (field.energy_fp64 / decode_energy_sums), the kinetic energy and the
    bond and angle virials; self_energy (not None) adds the electrostatic
    terms of PIC_Spectral."""
    V = e["V"]
    sigma = e["sigma"]
    means = e["means"]
    p1 = e["A"] + float((e["Q"] @ means + e["b"]) @ means)
    p2 = -sigma ** 2 * np.asarray(e["B"])
    w_elec = 0.0
    if self_energy is not None:
        p1 += e["C0"]
        p2 = p2 - sigma ** 2 * np.asarray(e["C"])
        w_elec = 0.5 * V * e["Eq"] - self_energy
    p_kin = 2.0 / (3.0 * V) * ke
    p0 = -(e["W"] + w_elec) / V
    p_bond = np.asarray(bond_pr, dtype=np.float64) / V
    p_angle = np.asarray(angle_pr, dtype=np.float64) / V
    p_dih = np.zeros(3)
    p_tot = p_kin + p0 + p1 + p2 + p_bond + p_angle + p_dih
    return np.array([p_kin, p0, p1, *p2, *p_bond, *p_angle, *p_dih, *p_tot])


def _host(x):
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return x
