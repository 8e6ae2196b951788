"""Differentiable hPF field energy: W(positions, chi, kappa, sigma).

The reference computes forces and energies only (hymd/field.py:152-200,
619-703); fitting chi to target structure needs gradients of the energy with
respect to the functional's parameters.  `field_energy` returns W as a torch
scalar whose backward pass runs the hand-written adjoint in libhpf_gb300.so
(hpf_field_adjoint):

  dW/dx_i      = m_t sum_g V_t(g) grad W_CIC(g - x_i),  V_t = H * (Q phi~)_t
  dW/dchi_ij   = S_ij / rho0                  (one parameter per pair i < j)
  dW/dkappa    = -1/(2 kappa^2 rho0) sum_g (sum_t phi~_t - a)^2 dV
  dW/dsigma    = -sigma sum_tj Q_tj sum_g phi~_j (-lap phi~_t) dV

with S_tj = sum_g phi~_t phi~_j dV, for the three functionals of
hymd/hamiltonian.py (DefaultWithChi :393-412, DefaultNoChi :259-260,
SquaredPhi :145-146), all of the form w = 1/2 phi~.Q.phi~ + b.phi~ + c with

  Q_ij = 1/(kappa rho0) + chi_ij/rho0 (i != j),  b_i = -a/(kappa rho0),
  c = a^2/(2 kappa rho0)          (SquaredPhi: a = 0, no chi).

The chi matrix is used symmetrised, chi_ij -> (chi_ij + chi_ji)/2, and its
diagonal is unused (the reference sums i < j only), so the returned gradient
is symmetric with G_ij = G_ji = S_ij / (2 rho0) and a zero diagonal: moving
one pair's chi by d (both entries) changes W by S_ij d / rho0.

dW/dx is the exact derivative of the discrete energy; the MD force (the
spectral readout of -grad V) equals -dW/dx only up to the difference
between the two discretisations of the gradient, which vanishes as the mesh
is refined (gradient_gap measures it).  field_energy(...,
reference_gradient=True) returns minus the MD force as the positions'
gradient instead, so that a loss differentiated through W follows the
reference's own forces.
"""
import numpy as np
import torch

from . import _lib

KINDS = ("DefaultWithChi", "DefaultNoChi", "SquaredPhi")


def functional_coefficients(kind, chi, kappa, rho0, a):
    """(Q, b, c) of the quadratic functional (numpy float64)."""
    if kind not in KINDS:
        raise NotImplementedError(f"no adjoint for functional {kind!r}")
    chi = np.asarray(chi, np.float64)
    T = chi.shape[0]
    inc = 1.0 / (kappa * rho0)
    Q = np.full((T, T), inc)
    if kind == "DefaultWithChi":
        cs = 0.5 * (chi + chi.T)
        off = ~np.eye(T, dtype=bool)
        Q[off] += cs[off] / rho0
    aa = 0.0 if kind == "SquaredPhi" else float(a)
    b = np.full(T, -aa * inc)
    c = 0.5 * aa * aa * inc
    return Q, b, c


def _set(pm, Q, b, c, sigma):
    _lib.call("hpf_ctx_set_functional", pm._h, _lib.dvec(Q.reshape(-1)), _lib.dvec(b), float(c),
              float(sigma))
    pm._functional = None  # the cached key no longer describes the context


def _energy(pm, pos, typ, masses, Q, b, c):
    T = pm.n_types
    out = torch.zeros(32, dtype=torch.float64, device=pm.device)
    _lib.call("hpf_energy_fp64", pm._h, _lib.ptr(pos), _lib.ptr(typ), pos.shape[0],
              _lib.dvec(masses), None, None, 0.0, _lib.ptr(out), _lib.stream_ptr())
    o = out.cpu().numpy()
    V = float(np.prod(pm.BoxSize))
    means = o[16:16 + T]
    return V * (0.5 * means @ Q @ means + b @ means + c) + 0.5 * V * o[0]


class _FieldEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, positions, chi, kappa, sigma, pm, types, masses, kind, rho0, a, ref_grad):
        k, s = float(kappa), float(sigma)
        Q, b, c = functional_coefficients(kind, chi.detach().cpu().numpy(), k, rho0, a)
        _set(pm, Q, b, c, s)
        W = _energy(pm, positions, types, masses, Q, b, c)
        ctx.pm, ctx.types, ctx.masses, ctx.kind = pm, types, masses, kind
        ctx.rho0, ctx.a, ctx.kappa, ctx.sigma = rho0, a, k, s
        ctx.Q, ctx.b, ctx.c = Q, b, c
        ctx.ref_grad = bool(ref_grad)
        ctx.chi_meta = (chi.dtype, chi.device)
        ctx.save_for_backward(positions)
        return torch.tensor(W, dtype=torch.float64, device=positions.device)

    @staticmethod
    def backward(ctx, gW):
        (positions,) = ctx.saved_tensors
        pm, T = ctx.pm, ctx.pm.n_types
        _set(pm, ctx.Q, ctx.b, ctx.c, ctx.sigma)
        need_x = ctx.needs_input_grad[0]
        need_p = any(ctx.needs_input_grad[1:4])
        grad_x = torch.empty_like(positions) if need_x else None
        P = T * (T + 1) // 2
        sums = torch.zeros(P + 1 + T, dtype=torch.float64, device=positions.device) if need_p \
            else None
        if need_x and ctx.ref_grad:
            # minus the MD force (the readout of the spectral gradient)
            _lib.call("hpf_field_step", pm._h, _lib.ptr(positions), _lib.ptr(ctx.types),
                      positions.shape[0], _lib.dvec(ctx.masses), _lib.ptr(grad_x), None, None,
                      None, _lib.stream_ptr())
            grad_x.neg_()
        if (need_x and not ctx.ref_grad) or need_p:
            _lib.call("hpf_field_adjoint", pm._h, _lib.ptr(positions), _lib.ptr(ctx.types),
                      positions.shape[0], _lib.dvec(ctx.masses),
                      _lib.ptr(grad_x) if (need_x and not ctx.ref_grad) else None,
                      _lib.ptr(sums), _lib.stream_ptr())
        g = float(gW.detach().item())
        out = [None] * 11
        if need_x:
            out[0] = grad_x * g
        if need_p:
            o = sums.cpu().numpy()
            V = float(np.prod(pm.BoxSize))
            means = o[P + 1:P + 1 + T]
            S = np.zeros((T, T))
            p = 0
            for t in range(T):
                for j in range(t, T):
                    S[t, j] = S[j, t] = o[p]
                    p += 1
            S = V * (S + np.outer(means, means))
            rho0, kappa = ctx.rho0, ctx.kappa
            aa = 0.0 if ctx.kind == "SquaredPhi" else float(ctx.a)
            dtype, dev = ctx.chi_meta
            if ctx.needs_input_grad[1]:
                G = np.zeros((T, T))
                if ctx.kind == "DefaultWithChi":
                    off = ~np.eye(T, dtype=bool)
                    G[off] = S[off] / (2.0 * rho0)
                out[1] = torch.as_tensor(G * g, dtype=dtype, device=dev)
            if ctx.needs_input_grad[2]:
                incomp = 0.5 * (S.sum() - 2.0 * aa * V * means.sum() + aa * aa * V) / rho0
                out[2] = torch.tensor(-incomp / kappa ** 2 * g, dtype=torch.float64)
            if ctx.needs_input_grad[3]:
                out[3] = torch.tensor(-ctx.sigma * V * o[P] * g, dtype=torch.float64)
        pm.check_errors()
        return tuple(out)


def field_energy(positions, types, pm, masses, chi, kappa, sigma, rho0, a,
                 kind="DefaultWithChi", reference_gradient=False):
    """W (FP64 torch scalar) of the current positions with the quadratic
    functional `kind` at (chi, kappa, sigma); differentiable with respect to
    positions (float32 CUDA (N,3)), chi ((T,T) tensor), kappa and sigma
    (0-d float64 tensors or floats).  reference_gradient: the positions'
    gradient is minus the MD force (hymd/field.py:152-200) instead of the
    exact dW/dx."""
    pos = _lib.require_cuda(positions, "positions", torch.float32)
    typ = types if types.dtype == torch.int32 else types.to(torch.int32)
    _lib.require_cuda(typ, "types", torch.int32, (pos.shape[0],))
    T = pm.n_types
    if not isinstance(chi, torch.Tensor):
        chi = torch.as_tensor(np.asarray(chi, np.float64))
    if tuple(chi.shape) != (T, T):
        raise ValueError(f"chi must be ({T}, {T})")
    if not isinstance(kappa, torch.Tensor):
        kappa = torch.tensor(float(kappa), dtype=torch.float64)
    if not isinstance(sigma, torch.Tensor):
        sigma = torch.tensor(float(sigma), dtype=torch.float64)
    m = [float(x) for x in masses] if masses is not None else [1.0] * T
    return _FieldEnergy.apply(pos, chi, kappa, sigma, pm, typ, m, kind, float(rho0), float(a),
                              bool(reference_gradient))


def gradient_gap(positions, types, pm, masses, chi, kappa, sigma, rho0, a,
                 kind="DefaultWithChi"):
    """Relative RMS difference between the MD field force F (hymd/field.py:
    152-200: the CIC readout of the spectral gradient of v_ext) and minus the
    exact derivative dW/dx of the discrete field energy, ||F + dW/dx|| /
    ||F||, at the given positions."""
    pos = _lib.require_cuda(positions, "positions", torch.float32).detach().clone()
    pos.requires_grad_(True)
    W = field_energy(pos, types, pm, masses, chi, kappa, sigma, rho0, a, kind)
    (g,) = torch.autograd.grad(W, pos)
    typ = types if types.dtype == torch.int32 else types.to(torch.int32)
    F = torch.empty_like(pos)
    m = [float(x) for x in masses] if masses is not None else [1.0] * pm.n_types
    _lib.call("hpf_field_step", pm._h, _lib.ptr(pos.detach()), _lib.ptr(typ), pos.shape[0],
              _lib.dvec(m), _lib.ptr(F), None, None, None, _lib.stream_ptr())
    d = (F.double() + g.double())
    return float(torch.sqrt((d ** 2).mean()) / torch.sqrt((F.double() ** 2).mean()))
