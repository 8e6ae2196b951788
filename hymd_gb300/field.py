"""Particle-field forces and energies on GB300 -- drop-in for hymd/field.py.

Same function names and positional signatures as the reference
(hymd/field.py:10-703); pmesh RealField / ComplexField objects become CUDA
torch tensors and the pmesh ParticleMesh becomes a `ParticleMesh` context
that owns the cuFFT plans.  Every numerical step runs in libhpf_gb300.so.

Grid layout: the lists returned by `initialize_pm` are views into stacked,
contiguous tensors -- phi is phi_all[t] of phi_all (T, n0, n1, n2),
force_on_grid[t][d] is force_all[t, d] of (T, 3, n0, n1, n2), complex fields
are complex64 (n0, n1, n2//2 + 1).  The stacked layout lets one kernel launch
serve all types; functions here accept only such stacks (ValueError otherwise).

`layouts` / `layout_q` arguments (pmesh domain layouts) are accepted and
ignored: one GPU holds the whole system.
"""
import numpy as np
import torch

from . import _lib
from .hamiltonian import quadratic_form

_REGISTRY = {}


class ParticleMesh:
    """Mesh context: geometry, box state, functional and cuFFT plans on the
    current CUDA device (replaces pmesh.pm.ParticleMesh)."""

    def __init__(self, mesh_size, box_size, n_types, device=None):
        n = np.asarray(mesh_size, dtype=np.int64).reshape(-1)
        if n.size == 1:
            n = np.repeat(n, 3)
        self.Nmesh = tuple(int(x) for x in n)
        self.n_types = int(n_types)
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self.BoxSize = np.asarray(box_size, dtype=np.float64).reshape(3).copy()
        self.M = int(np.prod(self.Nmesh))
        self.Mc = self.Nmesh[0] * self.Nmesh[1] * (self.Nmesh[2] // 2 + 1)
        handle = _lib.P()
        with torch.cuda.device(self.device):
            _lib.call("hpf_ctx_create", _lib.ctypes.byref(handle), self.Nmesh[0], self.Nmesh[1],
                      self.Nmesh[2], self.n_types, _lib.dvec(self.BoxSize))
        self._h = handle
        st = _lib.P()
        _lib.call("hpf_ctx_box_state", self._h, _lib.ctypes.byref(st))
        self.box_state_ptr = st.value
        self._functional = None
        self.ws = _lib.new_workspace(self.device)
        self.spec_raw = self.complex_field(self.n_types)
        self.spec_force = self.complex_field(3 * self.n_types)

    # -- allocation helpers -------------------------------------------------
    def real_field(self, *lead):
        return torch.zeros(*lead, *self.Nmesh, dtype=torch.float32, device=self.device)

    def complex_field(self, *lead):
        return torch.zeros(*lead, self.Nmesh[0], self.Nmesh[1], self.Nmesh[2] // 2 + 1,
                           dtype=torch.complex64, device=self.device)

    def create(self, kind, value=0.0):
        """pmesh-style single field."""
        f = self.real_field() if kind == "real" else self.complex_field()
        if value:
            f.fill_(value)
        return f

    def decompose(self, positions, smoothing=None):
        """Domain layouts are not needed on one GPU."""
        return None

    # -- state ----------------------------------------------------------------
    def set_box(self, box_size):
        self.BoxSize = np.asarray(box_size, dtype=np.float64).reshape(3).copy()
        _lib.call("hpf_ctx_set_box", self._h, _lib.dvec(self.BoxSize), _lib.stream_ptr())

    def box_tensor(self):
        """(3,) float64 device tensor aliasing the context box state (L)."""
        return _box_view(self)

    def set_functional(self, hamiltonian):
        Q, b, c, sigma = quadratic_form(hamiltonian, self.n_types)
        key = (Q.tobytes(), b.tobytes(), c, sigma)
        if key != self._functional:
            T = self.n_types
            if Q.shape != (T, T):
                raise ValueError(f"functional has {Q.shape[0]} types, mesh context has {T}")
            _lib.call("hpf_ctx_set_functional", self._h, _lib.dvec(Q.reshape(-1)), _lib.dvec(b),
                      float(c), float(sigma))
            self._functional = key
            self._functional_Q = Q
        return Q, b, c, sigma

    @property
    def spectral(self):
        """Transform path of the fused field step: "fused" (this library's
        shared-memory FFTs; default on power-of-two meshes) or "cufft"."""
        f, a = _lib.ctypes.c_int(0), _lib.ctypes.c_int(0)
        _lib.call("hpf_ctx_get_spectral", self._h, _lib.ctypes.byref(f), _lib.ctypes.byref(a))
        return "fused" if f.value else "cufft"

    @spectral.setter
    def spectral(self, path):
        if path not in ("fused", "cufft"):
            raise ValueError(f"spectral path {path!r}: 'fused' or 'cufft'")
        _lib.call("hpf_ctx_set_spectral", self._h, 1 if path == "fused" else 0)

    @property
    def spectral_available(self):
        f, a = _lib.ctypes.c_int(0), _lib.ctypes.c_int(0)
        _lib.call("hpf_ctx_get_spectral", self._h, _lib.ctypes.byref(f), _lib.ctypes.byref(a))
        return bool(a.value)

    @property
    def spectral_tile(self):
        """Columns per block of the fused k-space pass (4, 8 or 16; 0 without
        the fused path).  Forces do not depend on it; the energy sums only
        through their summation order."""
        w, m = _lib.ctypes.c_int(0), _lib.ctypes.c_int(0)
        _lib.call("hpf_ctx_get_spectral_tile", self._h, _lib.ctypes.byref(w),
                  _lib.ctypes.byref(m))
        return w.value

    @spectral_tile.setter
    def spectral_tile(self, width):
        _lib.call("hpf_ctx_set_spectral_tile", self._h, int(width))

    @property
    def spectral_tiles_allowed(self):
        w, m = _lib.ctypes.c_int(0), _lib.ctypes.c_int(0)
        _lib.call("hpf_ctx_get_spectral_tile", self._h, _lib.ctypes.byref(w),
                  _lib.ctypes.byref(m))
        return [x for x in (4, 8, 16) if m.value & x]

    def check_errors(self):
        code = _lib.ctypes.c_int(0)
        _lib.call("hpf_get_error", self._h, _lib.stream_ptr(), _lib.ctypes.byref(code))
        if code.value:
            raise _lib.HPFError("device check", code.value)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().hpf_ctx_destroy(h)
            except Exception:
                pass
            self._h = None


def _box_view(pm):
    """A (3,) float64 tensor over the device box state (no copy)."""
    if getattr(pm, "_box_t", None) is None:
        # wrap the raw device pointer: the first 3 doubles of the box state
        holder = _DevicePtrArray(pm.box_state_ptr, 3, pm.device)
        pm._box_t = holder.tensor
        pm._box_holder = holder
    return pm._box_t


class _DevicePtrArray:
    """Expose a library-owned device array as a torch tensor via DLPack-free
    __cuda_array_interface__ (lifetime tied to the owning context)."""

    def __init__(self, ptr, n, device):
        self.__cuda_array_interface__ = {
            "shape": (n,), "typestr": "<f8", "data": (int(ptr), False), "version": 2,
            "strides": None,
        }
        with torch.cuda.device(device):
            self.tensor = torch.as_tensor(self, device=device)


def _stack_base(lst, lead_shape, dtype, name):
    """Return the stacked tensor that the list elements are views of."""
    flat = []

    def walk(x):
        if isinstance(x, (list, tuple)):
            for y in x:
                walk(y)
        else:
            flat.append(x)

    walk(lst)
    first = flat[0]
    _lib.require_cuda(first, name + "[0]", dtype)
    per = first.numel() * first.element_size()
    for i, x in enumerate(flat):
        if x.dtype != dtype or x.data_ptr() != first.data_ptr() + i * per or not x.is_contiguous():
            raise ValueError(f"{name} must be views of one stacked tensor as created by "
                             "initialize_pm")
    base = torch.as_strided(first, (len(flat),) + tuple(first.shape),
                            (first.numel(),) + tuple(first.stride()))
    return base.reshape(tuple(lead_shape) + tuple(first.shape))


def initialize_pm(pmesh, config, comm=None):
    """hymd/field.py:10-149.  `pmesh` is ignored (may be None).

    Returns (pm, field_list, elec_common_list, coulomb_list) with the same
    nesting as the reference; fields are CUDA tensors (views of stacks).
    """
    T = config.n_types
    pm = ParticleMesh(config.mesh_size, config.box_size, T)
    phi_all = pm.real_field(T)
    phi_fourier_all = pm.complex_field(T)
    force_all = pm.real_field(T, 3)
    v_ext_fourier_all = pm.complex_field(4)
    v_ext_all = pm.real_field(T)
    phi_transfer_all = pm.complex_field(3)
    phi_lap_all = pm.real_field(T, 3)
    phi = [phi_all[t] for t in range(T)]
    phi_fourier = [phi_fourier_all[t] for t in range(T)]
    force_on_grid = [[force_all[t, d] for d in range(3)] for t in range(T)]
    v_ext_fourier = [v_ext_fourier_all[i] for i in range(4)]
    v_ext = [v_ext_all[t] for t in range(T)]
    phi_transfer = [phi_transfer_all[i] for i in range(3)]
    phi_laplacian = [[phi_lap_all[t, d] for d in range(3)] for t in range(T)]
    elec_common_list = [None, None, None, None]
    coulomb_list = []
    if config.coulombtype in ("PIC_Spectral", "PIC_Spectral_GPE"):
        phi_q = pm.real_field()
        phi_q_fourier = pm.complex_field()
        psi = pm.real_field()
        ef_all = pm.real_field(3)
        elec_common_list = [phi_q, phi_q_fourier, psi, [ef_all[d] for d in range(3)]]
    if config.coulombtype == "PIC_Spectral":
        eff_all = pm.complex_field(3)
        coulomb_list = [[eff_all[d] for d in range(3)], pm.complex_field()]
    elif config.coulombtype == "PIC_Spectral_GPE":
        # the 12 grids of the reference's GPE list (hymd/field.py:81-131), in
        # its order; phi_eps / phi_pol_prev / elec_field_contrib persist
        eta_all = pm.real_field(3)
        etaf_all = pm.complex_field(3)
        vbar_all = pm.real_field(T)
        vbarf_all = pm.complex_field(T)
        fme_all = pm.real_field(T, 3)
        fmef_all = pm.complex_field(T, 3)
        coulomb_list = [pm.real_field(), pm.complex_field(), [eta_all[d] for d in range(3)],
                        [etaf_all[d] for d in range(3)], pm.real_field(), pm.real_field(),
                        pm.real_field(), pm.real_field(), [vbar_all[t] for t in range(T)],
                        [vbarf_all[t] for t in range(T)],
                        [[fme_all[t, d] for d in range(3)] for t in range(T)],
                        [[fmef_all[t, d] for d in range(3)] for t in range(T)]]
        pm.gpe = dict(vbar=vbar_all, elec_field=ef_all)
    field_list = [phi, phi_fourier, force_on_grid, v_ext_fourier, v_ext, phi_transfer,
                  phi_laplacian]
    _REGISTRY[phi_all.data_ptr()] = pm
    pm.fields = dict(phi=phi_all, phi_fourier=phi_fourier_all, force=force_all,
                     v_ext=v_ext_all, phi_laplacian=phi_lap_all)
    return pm, field_list, elec_common_list, coulomb_list


def _pm_of(phi):
    pm = _REGISTRY.get(phi[0].data_ptr())
    if pm is None:
        raise ValueError("phi was not created by hymd_gb300.field.initialize_pm")
    return pm


def _masses(m, T):
    if m is None or len(m) == 0:
        return [1.0] * T
    return [float(x) for x in m]


def _types32(types, n):
    if types.dtype != torch.int32:
        types = types.to(torch.int32)
    return _lib.require_cuda(types.contiguous(), "types", torch.int32, (n,))


def update_field(phi, phi_laplacian, phi_transfer, layouts, force_mesh, hamiltonian, pm,
                 positions, types, config, v_ext, phi_fourier, v_ext_fourier, m,
                 compute_potential=False):
    """hymd/field.py:428-616.

    On return (as in the reference): phi[t] holds the filtered density
    phi~_t, phi_fourier[t] = H r2c(phi_t), force_mesh[t][d] = c2r(-i k_d H
    r2c(v_ext_t(phi~))) and, with compute_potential, v_ext[t] the filtered
    external potential.  v_ext_fourier is scratch in the reference and is not
    written here.
    """
    T = pm.n_types
    pos = _lib.require_cuda(positions, "positions", torch.float32)
    n = pos.shape[0]
    typ = _types32(types, n)
    phi_all = _stack_base(phi, (T,), torch.float32, "phi")
    phif_all = _stack_base(phi_fourier, (T,), torch.complex64, "phi_fourier")
    force_all = _stack_base(force_mesh, (T, 3), torch.float32, "force_mesh")
    pm.set_functional(hamiltonian)
    st = _lib.stream_ptr()
    masses = _lib.dvec(_masses(m, T))
    _lib.call("hpf_paint", pm._h, _lib.ptr(pos), _lib.ptr(typ), n, masses, _lib.ptr(phi_all), st)
    _lib.call("hpf_r2c", pm._h, _lib.ptr(phi_all), _lib.ptr(pm.spec_raw), T, st)
    v_k = pm.complex_field(T) if compute_potential else None
    _lib.call("hpf_kspace_force", pm._h, _lib.ptr(pm.spec_raw), _lib.ptr(pm.spec_force),
              _lib.ptr(phif_all), _lib.ptr(v_k), None, st)
    _lib.call("hpf_c2r", pm._h, _lib.ptr(pm.spec_force), _lib.ptr(force_all), 3 * T, st)
    _lib.call("hpf_c2r", pm._h, _lib.ptr(phif_all), _lib.ptr(phi_all), T, st)
    if compute_potential:
        vext_all = _stack_base(v_ext, (T,), torch.float32, "v_ext")
        _lib.call("hpf_c2r", pm._h, _lib.ptr(v_k), _lib.ptr(vext_all), T, st)
    pm.last_types = typ


def compute_field_force(layouts, r, force_mesh, force, types, n_types):
    """hymd/field.py:152-200: force[types == t, d] = readout(force_mesh[t][d])."""
    pos = _lib.require_cuda(r, "r", torch.float32)
    n = pos.shape[0]
    _lib.require_cuda(force, "force", torch.float32, (n, 3))
    force_all = _stack_base(force_mesh, (n_types, 3), torch.float32, "force_mesh")
    pm = _REGISTRY_FORCE.get(force_all.data_ptr())
    if pm is None:
        pm = _find_pm_for_force(force_all)
    typ = _types32(types, n)
    _lib.call("hpf_readout", pm._h, _lib.ptr(force_all), _lib.ptr(pos), _lib.ptr(typ), n,
              _lib.ptr(force), _lib.stream_ptr())


_REGISTRY_FORCE = {}


def _find_pm_for_force(force_all):
    for pm in _REGISTRY.values():
        if pm.fields["force"].data_ptr() == force_all.data_ptr():
            _REGISTRY_FORCE[force_all.data_ptr()] = pm
            return pm
    raise ValueError("force_mesh was not created by hymd_gb300.field.initialize_pm")


def energy_fp64(pm, positions, types, masses, hamiltonian, charges=None, type_charges=None,
                elec_factor=0.0):
    """FP64 energy and pressure sums of the current positions (hpf_energy_fp64).

    Returns dict(W, A, B[3], Eq, C0, C[3], means[T], V): W = V w(means) + V/2 A."""
    T = pm.n_types
    Q, b, c, sigma = pm.set_functional(hamiltonian)
    pos = _lib.require_cuda(positions, "positions", torch.float32)
    n = pos.shape[0]
    typ = _types32(types, n)
    q = None if charges is None else _lib.require_cuda(charges, "charges", torch.float32, (n,))
    out = torch.zeros(32, dtype=torch.float64, device=pm.device)
    qt = _lib.dvec(list(type_charges)) if type_charges is not None else None
    _lib.call("hpf_energy_fp64", pm._h, _lib.ptr(pos), _lib.ptr(typ), n,
              _lib.dvec(_masses(masses, T)), _lib.ptr(q), qt, float(elec_factor), _lib.ptr(out),
              _lib.stream_ptr())
    return decode_energy_sums(out.cpu().numpy(), Q, b, c, sigma, float(np.prod(pm.BoxSize)), T)


def decode_energy_sums(o, Q, b, c, sigma, V, T):
    """The dict of energy_fp64 from the host copy `o` of hpf_energy_fp64's
    double[32] output, for the functional (Q, b, c, sigma) and volume V."""
    means = np.array(o[16:16 + T], dtype=np.float64)
    W = V * (0.5 * means @ Q @ means + b @ means + c) + 0.5 * V * o[0]
    return dict(W=W, A=o[0], B=np.array(o[1:4]), Eq=o[4], C0=o[5], C=np.array(o[6:9]),
                means=means, V=V, Q=Q, b=b, sigma=sigma)


def compute_field_and_kinetic_energy(phi, phi_q, psi, velocity, hamiltonian, positions, types,
                                     v_ext, config, layouts, comm=None):
    """hymd/field.py:619-703 -> (field_energy, kinetic_energy, field_q_energy).

    W = sum_g w_0(phi~) dV and, with PIC_Spectral, W_elec = sum_g (phi_q psi /
    2 - E_self / V) dV are evaluated in FP64 for the given positions (the
    positions that produced phi in update_field): fixed-point densities ->
    FP64 FFT -> FP64 Parseval sums, with the k = 0 term from the exact means.
    The charges are those of the last update_field_force_q on this mesh.
    KE = m/2 sum v^2 (FP64 sum).
    """
    pm = _pm_of(phi)
    charges = None
    fac = 0.0
    if config.coulombtype == "PIC_Spectral":
        charges = getattr(pm, "pic_charges", None)
        if charges is None:
            raise ValueError("PIC_Spectral energy needs a preceding update_field_force_q")
        fac = config.coulomb_constant / config.dielectric_const
    e = energy_fp64(pm, positions, types, config.m, hamiltonian, charges=charges,
                    elec_factor=fac)
    vel = _lib.require_cuda(velocity, "velocity", torch.float32)
    _lib.call("hpf_sum_v2", _lib.ptr(vel), vel.shape[0], _lib.ptr(pm.ws), _lib.stream_ptr())
    ke = 0.5 * float(config.mass) * float(pm.ws[0])
    wq = 0.0
    if charges is not None:
        wq = 0.5 * e["V"] * e["Eq"] - float(config.self_energy or 0.0)
    return e["W"], ke, wq


def compute_self_energy_q(config, charges, comm=None):
    """hymd/field.py:203-238: k_e/eps sqrt(1/(2 pi sigma^2)) sum q^2 (FP64)."""
    q = _lib.require_cuda(charges, "charges", torch.float32)
    ws = _lib.new_workspace(q.device)
    _lib.call("hpf_sum_dot", _lib.ptr(q), _lib.ptr(q), q.numel(), _lib.ptr(ws), _lib.stream_ptr())
    pref = config.coulomb_constant / config.dielectric_const * np.sqrt(
        1.0 / (2.0 * np.pi * config.sigma * config.sigma))
    return float(pref * float(ws[0]))


def update_field_force_q(charges, phi_q, phi_q_fourier, psi, psi_fourier, elec_field_fourier,
                         elec_field, elec_forces, layout_q, hamiltonian, pm, positions, config):
    """hymd/field.py:241-403 (PIC_Spectral).

    Writes phi_q (painted q / dV), psi, elec_field[d], psi_fourier and
    elec_forces = q * readout(E).  phi_q_fourier and elec_field_fourier are
    transform scratch in the reference and are not written.
    """
    pos = _lib.require_cuda(positions, "positions", torch.float32)
    n = pos.shape[0]
    q = _lib.require_cuda(charges, "charges", torch.float32, (n,))
    _lib.require_cuda(elec_forces, "elec_forces", torch.float32, (n, 3))
    pm.set_functional(hamiltonian)
    ef_all = _stack_base(elec_field, (3,), torch.float32, "elec_field")
    fac = config.coulomb_constant / config.dielectric_const
    if getattr(pm, "pic_sums", None) is None:
        pm.pic_sums = torch.zeros(8, dtype=torch.float64, device=pm.device)
    _lib.call("hpf_pic_step", pm._h, _lib.ptr(pos), _lib.ptr(q), n, float(fac),
              _lib.ptr(elec_forces), _lib.ptr(phi_q), _lib.ptr(psi), _lib.ptr(ef_all),
              _lib.ptr(psi_fourier), _lib.ptr(pm.pic_sums), None, _lib.stream_ptr())
    # the charges of this evaluation, for the FP64 energy / pressure
    pm.pic_charges = q


_CONV_KINDS = {None: 0, "max_diff": 0, "csum": 1, "euclidean_norm": 2}


def update_field_force_q_GPE(conv_fun, phi, types, charges, phi_q, phi_q_fourier, phi_eps,
                             phi_eps_fourier, phi_eta, phi_eta_fourier, phi_pol_prev, phi_pol,
                             elec_field, elec_forces, elec_field_contrib, psi, Vbar_elec,
                             Vbar_elec_fourier, force_mesh_elec, force_mesh_elec_fourier,
                             hamiltonian, layout_q, layouts, pm, positions, config, comm=None):
    """hymd/field.py:764-1112 (PIC_Spectral_GPE) -> (Vbar_elec, phi_eps, elec_dot).

    `conv_fun` is the reference's convergence closure; the measure it stands
    for is taken from config.convergence_type (max_diff when unset, as
    hymd/main.py:141-165 does).  phi_eps and elec_field_contrib keep their
    contents between calls where the reference's masked divisions leave them
    (field.py:980,1066-1071); elec_forces is written in place.  psi,
    elec_field and Vbar_elec are filled; the Fourier grids of the argument
    list are scratch in the reference and not written.  The polarisation
    iteration starts from phi_pol_prev on every call and neither phi_pol_prev
    nor phi_pol is written: the reference rebinds both names locally
    (field.py:1010-1024), so its caller's grids keep their initial zeros and
    every solve starts cold.  The polarisation iteration runs as a CUDA
    graph whose loop test is evaluated on the device; the call synchronises
    once, at its end, to return the iteration count (pm.gpe_iterations)."""
    T = pm.n_types
    pos = _lib.require_cuda(positions, "positions", torch.float32)
    n = pos.shape[0]
    typ = _types32(types, n)
    q = _lib.require_cuda(charges, "charges", torch.float32, (n,))
    phi_all = _stack_base(phi, (T,), torch.float32, "phi")
    pm.set_functional(hamiltonian)
    kind = _CONV_KINDS.get(getattr(config, "convergence_type", None))
    if kind is None:
        raise ValueError(f"unknown convergence_type {config.convergence_type!r}")
    eps = [float(x) for x in config.dielectric_type]
    qt = [float(x) for x in (config.type_charges or [0.0] * T)]
    ef = pm.gpe["elec_field"] if hasattr(pm, "gpe") else pm.real_field(3)
    vb = pm.gpe["vbar"] if hasattr(pm, "gpe") else pm.real_field(T)
    dot = pm.real_field()
    pol = getattr(pm, "gpe_pol", None)
    if pol is None:
        pol = pm.gpe_pol = pm.real_field()
    pol.copy_(phi_pol_prev)  # the kernel iterates in place on this copy
    it = _lib.ctypes.c_int(0)
    _lib.call("hpf_gpe_step", pm._h, _lib.ptr(pos), _lib.ptr(typ), _lib.ptr(q), n,
              _lib.ptr(phi_all), _lib.dvec(eps), _lib.dvec(qt), float(config.coulomb_constant),
              float(config.conv_crit if config.conv_crit is not None else 1e-6),
              float(config.pol_mixing if config.pol_mixing is not None else 0.6), kind, 100,
              _lib.ptr(phi_eps), _lib.ptr(pol), _lib.ptr(elec_field_contrib),
              _lib.ptr(elec_forces), _lib.ptr(psi), _lib.ptr(ef), _lib.ptr(dot), _lib.ptr(vb),
              None, _lib.ctypes.byref(it), _lib.stream_ptr())
    for d in range(3):
        if elec_field[d].data_ptr() != ef[d].data_ptr():
            elec_field[d].copy_(ef[d])
    for t in range(T):
        if Vbar_elec[t].data_ptr() != vb[t].data_ptr():
            Vbar_elec[t].copy_(vb[t])
    pm.gpe_iterations = it.value
    return Vbar_elec, phi_eps, dot


def compute_field_energy_q_GPE(config, phi_eps, field_q_energy, dot_elec, comm=None):
    """hymd/field.py:706-761: dV eps0/2 sum(phi_eps |E|^2), in FP64."""
    V = float(np.prod(np.asarray(config.box_size, dtype=np.float64)))
    n = np.asarray(config.mesh_size).reshape(-1)
    cells = float(np.prod(np.full(3, n[0]) if n.size == 1 else n))
    eps_0 = 1.0 / (config.coulomb_constant * 4 * np.pi)
    return V / cells * (0.5 * eps_0) * float((phi_eps.double() * dot_elec.double()).sum())


def comp_laplacian(phi_fourier, phi_transfer, phi_laplacian, hamiltonian, config):
    """hymd/field.py:406-425: phi_laplacian[t][d] = c2r(-k_d^2 phi_fourier[t])."""
    pm = _pm_of_fourier(phi_fourier)
    T = pm.n_types
    phif_all = _stack_base(phi_fourier, (T,), torch.complex64, "phi_fourier")
    lap_all = _stack_base(phi_laplacian, (T, 3), torch.float32, "phi_laplacian")
    _lib.call("hpf_laplacian", pm._h, _lib.ptr(phif_all), _lib.ptr(lap_all), _lib.stream_ptr())


def _pm_of_fourier(phi_fourier):
    p = phi_fourier[0].data_ptr()
    for pm in _REGISTRY.values():
        if pm.fields["phi_fourier"].data_ptr() == p:
            return pm
    raise ValueError("phi_fourier was not created by hymd_gb300.field.initialize_pm")


def domain_decomposition(positions, pm, *args, molecules=None, bonds=None, topol=False,
                         verbose=0, comm=None):
    """hymd/field.py:1115-1178.  One GPU holds the whole system, so there is
    nothing to exchange: the arrays are returned unchanged."""
    return (positions, *args)


def paint_static(positions, types, masses, mesh_size, box_size, out=None, err=None):
    """Per-type CIC densities without a mesh context or any device allocation
    by the library (hpf_paint_static): the same grids as the paint inside
    `update_field` (hymd/field.py:573-575), bit for bit.

    For callers that own no `ParticleMesh` and may not allocate device memory
    themselves.  The library's scratch is a fixed 16 MiB static array per
    device, so n_types * prod(mesh_size) is limited to 2**21 cells
    (HPFError HPF_ERR_SCRATCH_LIMIT beyond).  Calls that overlap in time on
    one device race on that scratch.  `out` (float32, (T, n0, n1, n2)) and
    `err` (int32 device word) are caller-owned; without `out` a tensor is
    allocated here by torch.
    """
    pos = _lib.require_cuda(positions, "positions", torch.float32)
    n = pos.shape[0]
    typ = _types32(types, n)
    T = len(masses)
    n0, n1, n2 = (int(x) for x in mesh_size)
    if out is None:
        out = torch.empty((T, n0, n1, n2), dtype=torch.float32, device=pos.device)
    _lib.require_cuda(out, "out", torch.float32, (T, n0, n1, n2))
    _lib.call("hpf_paint_static", _lib.ptr(pos), _lib.ptr(typ), n, T, n0, n1, n2,
              _lib.dvec([float(x) for x in box_size]), _lib.dvec(_masses(masses, T)),
              _lib.ptr(out), _lib.ptr(err), _lib.stream_ptr())
    return out
