"""Reverse-mode gradients of hPF-MD trajectories (fitting chi to structure).

The reference integrates forces only (hymd/main.py:802-1169).  Here the same
rRESPA velocity-Verlet step is written with torch operations over two
differentiable force functions whose backward passes run hand-written
kernels in libhpf_gb300.so:

  * field force F(x, chi) -- forward hpf_field_step (paint -> r2c -> fused
    k-space -> c2r -> readout), backward hpf_field_force_vjp: the
    vector-Jacobian product with respect to the positions and the
    functional's matrix Q (hence chi);
  * electrostatic force of a charged system (PIC_Spectral,
    hymd/field.py:241-403) -- forward hpf_pic_step, backward
    hpf_pic_force_vjp (positions; the charges are constants);
  * bonded force F_b(x) (bonds, angles and four-body terms,
    hymd/compute_bond_forces.f90, compute_angle_forces.f90,
    compute_dihedral_forces.f90 with the CBT bending of
    dipole_reconstruction.f90) -- forward the fused plan's deterministic
    gather (hpf_respa_forces), backward hpf_bonded_hvp + hpf_dihedral_hvp
    (minus the Hessian of the bonded energy times the cotangent, by
    forward-mode dual arithmetic: the forces are minus the gradient of the
    energy, so the Jacobian is symmetric).  The one exception is the CBT
    bending force where the reference clamps sin(gamma) at 0.1
    (dipole_reconstruction.f90): there its force is not the gradient of its
    energy, and the product is that of the energy's Hessian;
  * the CSVR thermostat (hymd/thermostat.py:111-219) at the end of the outer
    step, when the RespaMD is coupled, with the random numbers of its table
    (row = step index), as torch operations.

A K-step loss is differentiated by torch autograd with the trajectory cut
into segments of ~sqrt(K) steps under torch.utils.checkpoint, so that only
the segment boundaries are stored and each segment is recomputed once in the
backward pass.  The loss provided is the mean squared deviation of the
time-averaged per-type density profile along z (linear binning, so that it
is differentiable in the positions) from a target profile.

Scope: NVE or NVT (CSVR); no barostat in the differentiated step;
PIC_Spectral electrostatics (not the GPE variant).
"""
import math

import numpy as np
import torch
from torch.utils.checkpoint import checkpoint

from . import _lib
from .adjoint import functional_coefficients


class ForceModel:
    """Everything the differentiable forces need, taken from a RespaMD
    (its mesh context, types, masses, topology and fused plan) plus the
    functional's parametrisation (kind, kappa, sigma, rho0, a)."""

    def __init__(self, md, kind="DefaultWithChi", kappa=None, sigma=None, rho0=None, a=None):
        if md.plan is None:
            raise ValueError("the bonded forward needs the fused plan (RespaMD(fused=True))")
        if md.perm is not None:
            raise ValueError("reverse mode works in the caller's bead order (no sort_particles)")
        if md.baro_args is not None:
            raise NotImplementedError("no barostat in the differentiated step")
        cfg = md.config
        self.md = md
        self.pm = md.pm
        self.kind = kind
        self.kappa = float(cfg.kappa if kappa is None else kappa)
        self.sigma = float(cfg.sigma if sigma is None else sigma)
        self.rho0 = float(cfg.rho0 if rho0 is None else rho0)
        self.a = float((cfg.a if cfg.a is not None else self.rho0) if a is None else a)
        self.T = md.T
        self.box = md.box
        self.box_f = md.box.float()
        self._key = None
        # PIC_Spectral electrostatics of a charged RespaMD
        self.charges = md.charges
        self.elec_factor = float(md.elec_factor) if md.charges is not None else 0.0
        # CSVR of a coupled RespaMD: its arguments and random table (host)
        self.thermo = md.thermo_args
        self.randoms = md.randoms.cpu().numpy() if self.thermo is not None else None
        self.group_masks = None
        if self.thermo is not None and md.group is not None:
            self.group_masks = [md.group == g for g in range(self.thermo.n_groups)]

    def set_chi(self, chi):
        Q, b, c = functional_coefficients(self.kind, chi.detach().cpu().numpy(), self.kappa,
                                          self.rho0, self.a)
        key = (Q.tobytes(), b.tobytes(), c, self.sigma)
        if key != self._key:
            _lib.call("hpf_ctx_set_functional", self.pm._h, _lib.dvec(Q.reshape(-1)),
                      _lib.dvec(b), float(c), float(self.sigma))
            self.pm._functional = None
            self._key = key


class _FieldForce(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, chi, model):
        model.set_chi(chi)
        md = model.md
        F = torch.empty_like(x)
        _lib.call("hpf_field_step", model.pm._h, _lib.ptr(x), _lib.ptr(md.types), md.n, md.masses,
                  _lib.ptr(F), None, None, None, _lib.stream_ptr())
        ctx.model = model
        ctx.chi_meta = (chi.dtype, chi.device, chi.detach().clone())
        ctx.save_for_backward(x)
        return F

    @staticmethod
    def backward(ctx, lam):
        (x,) = ctx.saved_tensors
        model = ctx.model
        md, T = model.md, model.T
        dtype, dev, chi = ctx.chi_meta
        model.set_chi(chi)
        g = torch.empty_like(x)
        need_chi = ctx.needs_input_grad[1]
        dQ = torch.zeros(T * T, dtype=torch.float64, device=x.device) if need_chi else None
        _lib.call("hpf_field_force_vjp", model.pm._h, _lib.ptr(x), _lib.ptr(md.types), md.n,
                  md.masses, _lib.ptr(lam.contiguous()), _lib.ptr(g), _lib.ptr(dQ),
                  _lib.stream_ptr())
        gchi = None
        if need_chi:
            dq = dQ.reshape(T, T)
            if model.kind == "DefaultWithChi":
                # Q_ij = (chi_ij + chi_ji) / (2 rho0) off the diagonal
                G = (dq + dq.T) / (2.0 * model.rho0)
                G.fill_diagonal_(0.0)
            else:
                G = torch.zeros_like(dq)
            gchi = G.to(dtype=dtype, device=dev)
        return g, gchi, None


class _BondedForce(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, model):
        md = model.md
        F = torch.zeros_like(x)
        _lib.call("hpf_respa_forces", md.plan, _lib.ptr(x), _lib.ptr(F), _lib.ptr(model.box),
                  None, _lib.ptr(md.err), _lib.stream_ptr())
        ctx.model = model
        ctx.save_for_backward(x)
        return F

    @staticmethod
    def backward(ctx, lam):
        (x,) = ctx.saved_tensors
        md = ctx.model.md
        t = md.topo
        out = torch.empty_like(x)
        lam = lam.contiguous()
        _lib.call("hpf_bonded_hvp", _lib.ptr(out), _lib.ptr(x), _lib.ptr(lam), md.n,
                  _lib.ptr(ctx.model.box), _lib.ptr(t.bond_a), _lib.ptr(t.bond_b),
                  _lib.ptr(t.bond_r0), _lib.ptr(t.bond_k), t.n_bonds, _lib.ptr(t.ang_a),
                  _lib.ptr(t.ang_b), _lib.ptr(t.ang_c), _lib.ptr(t.ang_t0), _lib.ptr(t.ang_k),
                  t.n_angles, _lib.ptr(md.err), _lib.stream_ptr())
        if t.n_dihedrals:
            _lib.call("hpf_dihedral_hvp", _lib.ptr(out), _lib.ptr(x), _lib.ptr(lam), md.n,
                      _lib.ptr(ctx.model.box), _lib.ptr(t.dih_a), _lib.ptr(t.dih_b),
                      _lib.ptr(t.dih_c), _lib.ptr(t.dih_d), _lib.ptr(t.dih_coeff),
                      _lib.ptr(t.dih_type), _lib.ptr(t.dih_last), t.n_dihedrals,
                      _lib.ptr(md.err), _lib.stream_ptr())
        return out, None


class _PicForce(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, model):
        md = model.md
        F = torch.empty_like(x)
        _lib.call("hpf_pic_step", model.pm._h, _lib.ptr(x), _lib.ptr(model.charges), md.n,
                  model.elec_factor, _lib.ptr(F), None, None, None, None, None, None,
                  _lib.stream_ptr())
        ctx.model = model
        ctx.save_for_backward(x)
        return F

    @staticmethod
    def backward(ctx, lam):
        (x,) = ctx.saved_tensors
        model = ctx.model
        g = torch.empty_like(x)
        _lib.call("hpf_pic_force_vjp", model.pm._h, _lib.ptr(x), _lib.ptr(model.charges),
                  model.md.n, model.elec_factor, _lib.ptr(lam.contiguous()), _lib.ptr(g),
                  _lib.stream_ptr())
        return g, None


def field_force(x, chi, model):
    """The slow force of the outer kicks: the field force, plus the
    PIC_Spectral electrostatic force of a charged system."""
    F = _FieldForce.apply(x, chi, model)
    if model.charges is not None:
        F = F + _PicForce.apply(x, model)
    return F


def bonded_force(x, model):
    if model.md.topo is None:
        return torch.zeros_like(x)
    return _BondedForce.apply(x, model)


def csvr(v, model, step):
    """The CSVR thermostat of outer step `step` (hymd/thermostat.py:167-219)
    as torch operations: per coupling group, in order, the kinetic energy
    (about the group's COM velocity with COM removal), the reference's
    alpha^2 from the group's (R, chi^2) draws of table row `step`, and the
    rescaling (of the group about its COM, or of every bead)."""
    a = model.thermo
    if (step + 1) % a.every:
        return v
    row = model.randoms[step * a.stride:(step + 1) * a.stride]
    m, c = model.md.mass, a.c
    for g in range(a.n_groups):
        sel = None if model.group_masks is None else model.group_masks[g]
        n_g = int(a.count[g])
        use_com = bool(a.remove_com) and n_g > 1
        if use_com:
            vg = v if sel is None else v[sel]
            com = vg.sum(0) / n_g
            K = 0.5 * m * ((vg - com) ** 2).sum()
        else:
            K = 0.5 * m * (v ** 2).sum()
        k_target = 1.5 * a.gas_constant * n_g * a.target_temperature
        nf = 3 * n_g
        R, S = float(row[a.offset + 2 * g]), float(row[a.offset + 2 * g + 1])
        q = k_target / (nf * K)
        alpha = torch.sqrt(c + (1.0 - c) * (S + R * R) * q + 2.0 * R * torch.sqrt(c * (1.0 - c) * q))
        if use_com:
            scaled = (v - com) * alpha + com
            v = scaled if sel is None else torch.where(sel[:, None], scaled, v)
        else:
            v = v * alpha
    return v


def respa_step(x, v, f_field, f_bond, chi, model, step=None):
    """One outer rRESPA step (hymd/main.py:802-887, 1143-1169) in torch
    operations: outer half kick, respa_inner x (half kick, drift, wrap,
    bonded forces, half kick), field forces, outer half kick, and the CSVR
    thermostat of outer step `step` when the RespaMD is coupled."""
    md = model.md
    m, dt, n_in = md.mass, md.dt, md.respa
    dto = n_in * dt
    v = v + (0.5 * dto / m) * f_field
    for _ in range(n_in):
        v = v + (0.5 * dt / m) * f_bond
        x = torch.remainder(x + dt * v, model.box_f)
        f_bond = bonded_force(x, model)
        v = v + (0.5 * dt / m) * f_bond
    f_field = field_force(x, chi, model)
    v = v + (0.5 * dto / m) * f_field
    if model.thermo is not None and step is not None:
        v = csvr(v, model, step)
    return x, v, f_field, f_bond


def z_profile(x, types, n_types, n_bins, box):
    """Per-type number density along z (beads / nm^3) with linear binning
    onto bin centres (periodic), differentiable in the positions."""
    Lz = box[2]
    s = x[:, 2] * (n_bins / Lz) - 0.5
    i0 = torch.floor(s).detach()
    f = s - i0
    i0 = i0.long() % n_bins
    i1 = (i0 + 1) % n_bins
    flat = torch.zeros(n_types * n_bins, dtype=x.dtype, device=x.device)
    t = types.long()
    flat = flat.index_add(0, t * n_bins + i0, 1.0 - f)
    flat = flat.index_add(0, t * n_bins + i1, f)
    vol = box[0] * box[1] * Lz / n_bins
    return flat.reshape(n_types, n_bins) / vol


def profile_loss(x0, v0, chi, model, n_steps, target, n_bins=100, segment=None, step0=0):
    """MSE between the z-density profile averaged over n_steps outer steps
    and `target` (n_types, n_bins), differentiable in x0, v0 and chi; the
    trajectory is checkpointed every `segment` steps (default ceil(sqrt(K))).
    step0: outer step index of the first step (the thermostat's table row)."""
    md = model.md
    seg = segment or max(1, int(math.ceil(math.sqrt(n_steps))))
    box = [float(b) for b in model.box.cpu()]
    types = md.types
    x, v = x0, v0
    f_field = field_force(x, chi, model)
    f_bond = bonded_force(x, model)

    def run(k, s0, x, v, f_field, f_bond, chi):
        acc = torch.zeros((model.T, n_bins), dtype=x.dtype, device=x.device)
        for i in range(k):
            x, v, f_field, f_bond = respa_step(x, v, f_field, f_bond, chi, model, s0 + i)
            acc = acc + z_profile(x, types, model.T, n_bins, box)
        return x, v, f_field, f_bond, acc

    total = torch.zeros((model.T, n_bins), dtype=x.dtype, device=x.device)
    done = 0
    while done < n_steps:
        k = min(seg, n_steps - done)
        x, v, f_field, f_bond, acc = checkpoint(run, k, step0 + done, x, v, f_field, f_bond,
                                                chi, use_reentrant=False)
        total = total + acc
        done += k
    prof = total / n_steps
    return torch.mean((prof - target) ** 2), prof
