"""Plain-torch FP64 restatement of the field and bonded forces, written so that
torch autograd can differentiate it (test infrastructure only: the reference
gradients for the hand-written reverse-mode kernels).

Same conventions as oracle/field.py (pmesh's CIC nodes at x = i h, r2c
normalised by 1/M, gradient wavevector with the Nyquist index at zero, filter
on the full |k|^2):
  field force   hymd/field.py:152-200, 428-616 (update_field, compute_field_force)
  bond force    hymd/compute_bond_forces.f90:45-61
  angle force   hymd/compute_angle_forces.f90:58-92
  PIC force     hymd/field.py:356-403 (update_field_force_q, PIC_Spectral)
  four-body     hymd/compute_dihedral_forces.f90:61-134 (cosine series of
                rows 0/1 and 2/3, type 2 improper) with the CBT bending
                energy of hymd/dipole_reconstruction.f90:50-106
The forces are minus the autograd gradient of the energies for the bonded
terms, and the explicit spectral-gradient readout for the field.
"""
import math

import numpy as np
import torch


def _kgrids(n, box, device):
    kx = 2 * math.pi / box[0] * torch.fft.fftfreq(n[0], 1.0 / n[0], dtype=torch.float64,
                                                   device=device)
    ky = 2 * math.pi / box[1] * torch.fft.fftfreq(n[1], 1.0 / n[1], dtype=torch.float64,
                                                   device=device)
    kz = 2 * math.pi / box[2] * torch.arange(n[2] // 2 + 1, dtype=torch.float64, device=device)
    kx, ky, kz = kx[:, None, None], ky[None, :, None], kz[None, None, :]
    k2 = kx * kx + ky * ky + kz * kz
    gx, gy, gz = kx.clone(), ky.clone(), kz.clone()
    if n[0] % 2 == 0:
        gx[n[0] // 2] = 0.0
    if n[1] % 2 == 0:
        gy[:, n[1] // 2] = 0.0
    if n[2] % 2 == 0:
        gz[:, :, n[2] // 2] = 0.0
    return k2, (gx, gy, gz)


def _cic(x, n, box):
    """Corner indices (8, N) into the flat mesh and weights (8, N), the
    weights differentiable in x."""
    nn = torch.tensor(n, dtype=torch.float64, device=x.device)
    L = torch.tensor(box, dtype=torch.float64, device=x.device)
    s = x * (nn / L)
    i0 = torch.floor(s).detach()
    f = s - i0
    i0 = i0.long()
    idx, w = [], []
    for a in (0, 1):
        for b in (0, 1):
            for c in (0, 1):
                ix = (i0[:, 0] + a) % n[0]
                iy = (i0[:, 1] + b) % n[1]
                iz = (i0[:, 2] + c) % n[2]
                idx.append((ix * n[1] + iy) * n[2] + iz)
                wa = f[:, 0] if a else 1.0 - f[:, 0]
                wb = f[:, 1] if b else 1.0 - f[:, 1]
                wc = f[:, 2] if c else 1.0 - f[:, 2]
                w.append(wa * wb * wc)
    return torch.stack(idx), torch.stack(w)


def field_force(x, types, n_types, masses, mesh, box, Q, sigma):
    """F (N,3) FP64 of the quadratic functional with matrix Q (T,T); x, Q may
    require grad."""
    n = tuple(int(v) for v in mesh)
    M = n[0] * n[1] * n[2]
    dV = float(np.prod(box)) / M
    idx, w = _cic(x, n, box)
    t = types.long()
    m = torch.as_tensor(masses, dtype=torch.float64, device=x.device)[t]
    flat = torch.zeros(n_types * M, dtype=torch.float64, device=x.device)
    flat = flat.index_add(0, (t[None, :] * M + idx).reshape(-1), (w * (m / dV)[None, :]).reshape(-1))
    phi = flat.reshape(n_types, *n)
    Phi = torch.fft.rfftn(phi, dim=(1, 2, 3))
    k2, g = _kgrids(n, box, x.device)
    H2 = torch.exp(-sigma * sigma * k2)
    QPhi = torch.einsum("tj,jxyz->txyz", Q.to(torch.complex128), Phi) * H2
    E = [torch.fft.irfftn(-1j * g[d] * QPhi, s=n, dim=(1, 2, 3)).reshape(n_types, M)
         for d in range(3)]
    F = []
    for d in range(3):
        Ed = E[d][t[None, :].expand(8, -1), idx]
        F.append((w * Ed).sum(0))
    return torch.stack(F, 1)


def pic_force(x, charges, mesh, box, sigma, elec_factor):
    """PIC_Spectral electrostatic force (hymd/field.py:356-403) in FP64:
    rho = CIC paint of q / dV, psi(k) = 4 pi f H rho(k) / k^2 (k = 0: k^2 =
    1), E_d = irfft(-i k'_d psi), F_i = q_i sum W E; x may require grad."""
    n = tuple(int(v) for v in mesh)
    M = n[0] * n[1] * n[2]
    dV = float(np.prod(box)) / M
    idx, w = _cic(x, n, box)
    q = torch.as_tensor(charges, dtype=torch.float64, device=x.device)
    flat = torch.zeros(M, dtype=torch.float64, device=x.device)
    flat = flat.index_add(0, idx.reshape(-1), (w * (q / dV)[None, :]).reshape(-1))
    R = torch.fft.rfftn(flat.reshape(n))
    k2, g = _kgrids(n, box, x.device)
    H = torch.exp(-0.5 * sigma * sigma * k2)
    k2z = k2.clone()
    k2z[0, 0, 0] = 1.0
    psi = 4.0 * math.pi * elec_factor * H * R / k2z
    F = []
    for d in range(3):
        Ed = torch.fft.irfftn(-1j * g[d] * psi, s=n).reshape(M)
        F.append(q * (w * Ed[idx]).sum(0))
    return torch.stack(F, 1)


def _min_image(r, box):
    L = torch.tensor(box, dtype=r.dtype, device=r.device)
    return r - L * torch.round(r / L)


def _series(c_row, d_row, phi):
    """sum_n c_n (1 + cos(n phi - d_n)), n = 0..4 (dipole_reconstruction.f90:37-48)."""
    n = torch.arange(5, dtype=phi.dtype, device=phi.device)
    return (c_row * (1.0 + torch.cos(n * phi[:, None] - d_row))).sum(1)


def dihedral_energy(x, box, dihedrals):
    """E of the four-body terms (a, b, c, d, coeff (D, 6, 5), type, last):
    type 0 the cosine series of rows 0/1 (+ rows 2/3 where both are
    non-zero), type 1 that plus the CBT bending 1/2 K(phi) (gamma -
    gamma_0(phi))^2 of the angle at b (and at c for the chain's last term),
    K the series of rows 4/5 and gamma_0 = 1.85 - 0.227 cos(phi - 0.785),
    type 2 the improper 1/2 k (phi - phi_0)^2 (row 0: phi_0, k)."""
    a, b, c, d, coeff, dtype, last = dihedrals
    f = _min_image(x[a] - x[b], box)
    g = _min_image(x[b] - x[c], box)
    h = _min_image(x[d] - x[c], box)
    v = torch.cross(f, g, dim=1)
    w = torch.cross(h, g, dim=1)
    gn = torch.linalg.norm(g, dim=1)
    phi = torch.atan2((w * f).sum(1) * gn, (v * w).sum(1))
    cf = coeff.to(x.dtype)
    e = _series(cf[:, 0], cf[:, 1], phi)
    second = (cf[:, 2] != 0).any(1) & (cf[:, 3] != 0).any(1)
    e = e + torch.where(second, _series(cf[:, 2], cf[:, 3], phi), torch.zeros_like(phi))
    E = (e * ((dtype == 0) | (dtype == 1)).to(x.dtype)).sum()
    K = _series(cf[:, 4], cf[:, 5], phi)
    # 0.785 as the single-precision literal of the Fortran
    gamma_0 = 1.85 - 0.227 * torch.cos(phi - float(np.float32(0.785)))

    def bend(rab, rcb):
        cg = (rab * rcb).sum(1) / (torch.linalg.norm(rab, dim=1) * torch.linalg.norm(rcb, dim=1))
        return 0.5 * K * (torch.acos(cg) - gamma_0) ** 2

    cbt = (dtype == 1).to(x.dtype)
    E = E + (bend(f, -g) * cbt).sum() + (bend(g, h) * cbt * (last == 1).to(x.dtype)).sum()
    imp = (dtype == 2).to(x.dtype)
    E = E + (0.5 * cf[:, 0, 1] * (phi - cf[:, 0, 0]) ** 2 * imp).sum()
    return E


def bonded_energy(x, box, bonds=None, angles=None, dihedrals=None):
    """E of harmonic bonds (a, b, r0, k), angles (a, b, c, t0, k) and the
    four-body terms (dihedral_energy)."""
    E = x.new_zeros(())
    if dihedrals is not None and len(dihedrals[0]):
        E = E + dihedral_energy(x, box, dihedrals)
    if bonds is not None and len(bonds[0]):
        a, b, r0, k = bonds
        r = _min_image(x[b] - x[a], box)
        d = torch.linalg.norm(r, dim=1)
        E = E + 0.5 * (k * (d - r0) ** 2).sum()
    if angles is not None and len(angles[0]):
        a, b, c, t0, k = angles
        ra = _min_image(x[a] - x[b], box)
        rc = _min_image(x[c] - x[b], box)
        ea = ra / torch.linalg.norm(ra, dim=1, keepdim=True)
        ec = rc / torch.linalg.norm(rc, dim=1, keepdim=True)
        th = torch.atan2(torch.linalg.norm(torch.cross(ea, ec, dim=1), dim=1), (ea * ec).sum(1))
        E = E + 0.5 * (k * (th - t0) ** 2).sum()
    return E


def bonded_force(x, box, bonds=None, angles=None, create_graph=True, dihedrals=None):
    if not x.requires_grad:
        x = x.detach().requires_grad_(True)
    E = bonded_energy(x, box, bonds, angles, dihedrals)
    (g,) = torch.autograd.grad(E, x, create_graph=create_graph)
    return -g
