"""Reverse mode through the forces and the rRESPA trajectory
(hymd_gb300.reverse) against a plain-torch FP64 reference differentiated by
torch autograd (oracle/torch_field.py), and that reference against FP64
central finite differences.

Tolerances: force vector-Jacobian products within 1e-4 relative RMS of the
FP64 autograd values (FP32 kernels); the K-step gradient of the profile loss
with respect to chi within 2e-3 relative (FP32 trajectory against FP64); the
FP64 reference gradient within 1e-5 of its central finite difference.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import torch_field as tf  # noqa: E402


def rel_rms(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def _membrane(respa_inner=3):
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    s = systems.lipid_membrane(seed=8, n_lipids=60, n_water=900, box=5.6, mesh=20)
    cfg = s["config"]
    cfg.respa_inner = respa_inner
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, get_hamiltonian(cfg),
                 topology=s["topology"], max_block_beads=36)
    names = cfg.unique_names
    T = cfg.n_types
    chi = np.zeros((T, T))
    for c in cfg.chi:
        i, j = names.index(c.atom_1), names.index(c.atom_2)
        chi[i, j] = chi[j, i] = c.interaction_energy
    return s, cfg, md, chi


def _Q_torch(chi, kappa, rho0):
    T = chi.shape[0]
    off = 1.0 - torch.eye(T, dtype=torch.float64, device=chi.device)
    return 1.0 / (kappa * rho0) + 0.5 * (chi + chi.T) * off / rho0


def test_field_force_vjp_matches_torch_autograd():
    from hymd_gb300 import _lib
    from hymd_gb300.reverse import ForceModel
    s, cfg, md, chi = _membrane()
    model = ForceModel(md)
    chi_t = torch.tensor(chi, dtype=torch.float64)
    model.set_chi(chi_t)
    rng = np.random.default_rng(1)
    lam = torch.tensor(rng.normal(size=(md.n, 3)), dtype=torch.float32, device="cuda")
    g = torch.empty_like(md.r)
    dQ = torch.zeros(md.T * md.T, dtype=torch.float64, device="cuda")
    _lib.call("hpf_field_force_vjp", md.pm._h, _lib.ptr(md.r), _lib.ptr(md.types), md.n,
              md.masses, _lib.ptr(lam), _lib.ptr(g), _lib.ptr(dQ), _lib.stream_ptr())
    x = md.r.double().clone().requires_grad_(True)
    Q = _Q_torch(chi_t.cuda(), model.kappa, model.rho0).detach().requires_grad_(True)
    F = tf.field_force(x, md.types, md.T, list(cfg.m), cfg.mesh(), list(cfg.box()), Q,
                       model.sigma)
    # the forward agrees first
    F32 = torch.empty_like(md.r)
    _lib.call("hpf_field_step", md.pm._h, _lib.ptr(md.r), _lib.ptr(md.types), md.n, md.masses,
              _lib.ptr(F32), None, None, None, _lib.stream_ptr())
    assert rel_rms(F32.cpu().numpy(), F.detach().cpu().numpy()) < 1e-5
    (lam.double() * F).sum().backward()
    assert rel_rms(g.cpu().numpy(), x.grad.cpu().numpy()) < 1e-4
    assert rel_rms(dQ.cpu().numpy(), Q.grad.reshape(-1).cpu().numpy()) < 1e-4
    md.check_errors()


def test_bonded_hvp_matches_torch_double_backward():
    from hymd_gb300 import _lib
    s, cfg, md, chi = _membrane()
    t = md.topo
    rng = np.random.default_rng(2)
    lam = torch.tensor(rng.normal(size=(md.n, 3)), dtype=torch.float32, device="cuda")
    out = torch.empty_like(md.r)
    _lib.call("hpf_bonded_hvp", _lib.ptr(out), _lib.ptr(md.r), _lib.ptr(lam), md.n,
              _lib.ptr(md.box), _lib.ptr(t.bond_a), _lib.ptr(t.bond_b), _lib.ptr(t.bond_r0),
              _lib.ptr(t.bond_k), t.n_bonds, _lib.ptr(t.ang_a), _lib.ptr(t.ang_b),
              _lib.ptr(t.ang_c), _lib.ptr(t.ang_t0), _lib.ptr(t.ang_k), t.n_angles,
              _lib.ptr(md.err), _lib.stream_ptr())
    bonds = (t.bond_a.long(), t.bond_b.long(), t.bond_r0.double(), t.bond_k.double())
    angles = (t.ang_a.long(), t.ang_b.long(), t.ang_c.long(), t.ang_t0.double(),
              t.ang_k.double())
    x = md.r.double().clone().requires_grad_(True)
    Fb = tf.bonded_force(x, list(cfg.box()), bonds, angles, create_graph=True)
    (hv,) = torch.autograd.grad((Fb * lam.double()).sum(), x)
    assert rel_rms(out.cpu().numpy(), hv.cpu().numpy()) < 1e-4
    md.check_errors()


def _torch_loss(x0, v0, chi, md, cfg, model, K, target, n_bins, bonds, angles, dihedrals=None,
                thermo=None, charges=None):
    """The same rRESPA trajectory and profile loss with the FP64 torch forces
    (four-body terms when given) and, with thermo = (args, random table),
    the CSVR of each outer step in FP64."""
    from hymd_gb300.reverse import z_profile
    box = list(cfg.box())
    L = torch.tensor(box, dtype=torch.float64, device=x0.device)
    Q = _Q_torch(chi, model.kappa, model.rho0)
    m, dt, n_in = md.mass, md.dt, md.respa
    dto = n_in * dt

    def ff(x):
        F = tf.field_force(x, md.types, md.T, list(cfg.m), cfg.mesh(), box, Q, model.sigma)
        if charges is not None:
            F = F + tf.pic_force(x, charges, cfg.mesh(), box, model.sigma, model.elec_factor)
        return F

    def fb(x):
        return tf.bonded_force(x, box, bonds, angles, create_graph=True, dihedrals=dihedrals)

    x, v = x0, v0
    f_field, f_bond = ff(x), fb(x)
    acc = 0.0
    for step in range(K):
        v = v + (0.5 * dto / m) * f_field
        for _ in range(n_in):
            v = v + (0.5 * dt / m) * f_bond
            x = torch.remainder(x + dt * v, L)
            f_bond = fb(x)
            v = v + (0.5 * dt / m) * f_bond
        f_field = ff(x)
        v = v + (0.5 * dto / m) * f_field
        if thermo is not None:
            v = _csvr64(v, m, step, *thermo)
        acc = acc + z_profile(x, md.types, md.T, n_bins, box)
    prof = acc / K
    return torch.mean((prof - target) ** 2)


def _csvr64(v, m, step, a, table):
    """thermostat.py:167-219 for one coupling group with COM removal, FP64."""
    row = table[step * a.stride:(step + 1) * a.stride]
    R, S = float(row[a.offset]), float(row[a.offset + 1])
    n = v.shape[0]
    com = v.sum(0) / n
    K = 0.5 * m * ((v - com) ** 2).sum()
    q = 1.5 * a.gas_constant * n * a.target_temperature / (3 * n * K)
    c = a.c
    alpha = torch.sqrt(c + (1 - c) * (S + R * R) * q + 2 * R * torch.sqrt(c * (1 - c) * q))
    return (v - com) * alpha + com


def test_profile_loss_gradient_matches_fp64_autograd_and_finite_differences():
    from hymd_gb300.reverse import ForceModel, profile_loss
    s, cfg, md, chi = _membrane()
    model = ForceModel(md)
    K, n_bins = 4, 20
    rng = np.random.default_rng(3)
    target = torch.tensor(rng.uniform(0.0, 3.0, size=(md.T, n_bins)), dtype=torch.float32,
                          device="cuda")
    chi_t = torch.tensor(chi, dtype=torch.float32, device="cuda", requires_grad=True)
    loss, _ = profile_loss(md.r.clone(), md.v.clone(), chi_t, model, K, target, n_bins=n_bins,
                           segment=2)
    loss.backward()
    g = chi_t.grad.double().cpu().numpy()
    t = md.topo
    bonds = (t.bond_a.long(), t.bond_b.long(), t.bond_r0.double(), t.bond_k.double())
    angles = (t.ang_a.long(), t.ang_b.long(), t.ang_c.long(), t.ang_t0.double(),
              t.ang_k.double())
    chi64 = torch.tensor(chi, dtype=torch.float64, device="cuda", requires_grad=True)
    args = (md, cfg, model, K, target.double(), n_bins, bonds, angles)
    x0, v0 = md.r.double(), md.v.double()
    L64 = _torch_loss(x0, v0, chi64, *args)
    L64.backward()
    g64 = chi64.grad.cpu().numpy()
    assert float(loss.detach()) == pytest.approx(float(L64.detach()), rel=1e-4)
    pairs = [(i, j) for i in range(md.T) for j in range(i + 1, md.T) if chi[i, j] != 0]
    got = np.array([g[i, j] + g[j, i] for i, j in pairs])
    want = np.array([g64[i, j] + g64[j, i] for i, j in pairs])
    assert rel_rms(got, want) < 2e-3
    # the FP64 reference itself against a central finite difference (one pair)
    i, j = pairs[0]
    h = 1e-3
    with torch.no_grad():
        cp, cm = chi64.detach().clone(), chi64.detach().clone()
        cp[i, j] += h
        cp[j, i] += h
        cm[i, j] -= h
        cm[j, i] -= h
    fd = (float(_torch_loss(x0, v0, cp, *args).detach())
          - float(_torch_loss(x0, v0, cm, *args).detach())) / (2 * h)
    assert want[0] == pytest.approx(fd, rel=1e-5)
    md.check_errors()


def _peptides(charged=False):
    """Peptide chains with CBT four-body terms (with charges: the side-chain
    and counter-ion charges of the recipe); no CBT angle near the
    reference's sin(gamma) = 0.1 clamp (where its force is not the gradient
    of its energy)."""
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    s = systems.charged_peptides(seed=22, n_chains=10, n_res=12, n_total=2500, box=6.0, mesh=24)
    cfg = s["config"]
    cfg.respa_inner = 3
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, get_hamiltonian(cfg),
                 topology=s["topology"], max_block_beads=36,
                 charges=s["charges"] if charged else None)
    names = cfg.unique_names
    T = cfg.n_types
    chi = np.zeros((T, T))
    for c in cfg.chi:
        i, j = names.index(c.atom_1), names.index(c.atom_2)
        chi[i, j] = chi[j, i] = c.interaction_energy
    return s, cfg, md, chi


def _dihedral_tuple(t, dtype=None):
    return (t.dih_a.long(), t.dih_b.long(), t.dih_c.long(), t.dih_d.long(),
            t.dih_coeff.double(), (t.dih_type if dtype is None else dtype).long(),
            t.dih_last.long())


def _min_sin_gamma(x, box, t):
    L = torch.tensor(box, dtype=torch.float64, device=x.device)
    mi = lambda r: r - L * torch.round(r / L)  # noqa: E731
    a, b, c, d = t.dih_a.long(), t.dih_b.long(), t.dih_c.long(), t.dih_d.long()
    out = []
    for p, q, r, use in ((a, b, c, t.dih_type == 1), (b, c, d, (t.dih_type == 1) & (t.dih_last == 1))):
        ra, rc = mi(x[p] - x[q]), mi(x[r] - x[q])
        cg = (ra * rc).sum(1) / (ra.norm(dim=1) * rc.norm(dim=1))
        sg = torch.sqrt(torch.clamp(1 - cg * cg, min=0.0))
        out.append(sg[use])
    return float(torch.cat(out).min())


def test_dihedral_hvp_matches_torch_double_backward():
    """hpf_dihedral_hvp (forward-mode duals over the four-body force) against
    the FP64 torch energy's double backward, for the cosine series (type 0),
    the cosine series with CBT bending (type 1, the chain's last term with
    the second bend) and the improper (type 2); the forces first against
    the per-term kernel."""
    from hymd_gb300 import _lib
    s, cfg, md, chi = _peptides()
    t = md.topo
    box = list(cfg.box())
    x64 = md.r.double()
    assert _min_sin_gamma(x64, box, t) > 0.2
    nd = t.n_dihedrals
    dtype = t.dih_type.clone()
    dtype[0::5] = 0
    dtype[3::7] = 2
    dih = _dihedral_tuple(t, dtype)
    # the force kernel against minus the torch energy gradient
    F = torch.zeros_like(md.r)
    out = _lib.new_workspace()
    _lib.call("hpf_dihedrals", _lib.ptr(F), _lib.ptr(md.r), md.n, None, None, _lib.ptr(md.box),
              _lib.ptr(t.dih_a), _lib.ptr(t.dih_b), _lib.ptr(t.dih_c), _lib.ptr(t.dih_d),
              _lib.ptr(t.dih_coeff), _lib.ptr(dtype), _lib.ptr(t.dih_last), nd, 0,
              _lib.ptr(out), _lib.ptr(md.err), _lib.stream_ptr())
    x = x64.clone().requires_grad_(True)
    Ft = tf.bonded_force(x, box, dihedrals=dih, create_graph=True)
    assert rel_rms(F.cpu().numpy(), Ft.detach().cpu().numpy()) < 1e-5
    rng = np.random.default_rng(4)
    lam = torch.tensor(rng.normal(size=(md.n, 3)), dtype=torch.float32, device="cuda")
    hv_gpu = torch.zeros_like(md.r)
    _lib.call("hpf_dihedral_hvp", _lib.ptr(hv_gpu), _lib.ptr(md.r), _lib.ptr(lam), md.n,
              _lib.ptr(md.box), _lib.ptr(t.dih_a), _lib.ptr(t.dih_b), _lib.ptr(t.dih_c),
              _lib.ptr(t.dih_d), _lib.ptr(t.dih_coeff), _lib.ptr(dtype), _lib.ptr(t.dih_last),
              nd, _lib.ptr(md.err), _lib.stream_ptr())
    (hv,) = torch.autograd.grad((Ft * lam.double()).sum(), x)
    assert rel_rms(hv_gpu.cpu().numpy(), hv.cpu().numpy()) < 1e-4
    md.check_errors()


def test_profile_loss_gradient_with_dihedrals_and_csvr():
    """The K-step chi gradient through a peptide trajectory with CBT
    four-body terms and the CSVR thermostat in every outer step, against
    the FP64 torch trajectory (autograd) and that against a central finite
    difference."""
    from hymd_gb300.reverse import ForceModel, profile_loss
    s, cfg, md, chi = _peptides()
    md.couple(thermostat=True, seed=7, n_steps=50)
    model = ForceModel(md)
    K, n_bins = 4, 20
    rng = np.random.default_rng(5)
    target = torch.tensor(rng.uniform(0.0, 3.0, size=(md.T, n_bins)), dtype=torch.float32,
                          device="cuda")
    chi_t = torch.tensor(chi, dtype=torch.float32, device="cuda", requires_grad=True)
    loss, _ = profile_loss(md.r.clone(), md.v.clone(), chi_t, model, K, target, n_bins=n_bins,
                           segment=2)
    loss.backward()
    g = chi_t.grad.double().cpu().numpy()
    t = md.topo
    bonds = (t.bond_a.long(), t.bond_b.long(), t.bond_r0.double(), t.bond_k.double())
    angles = (t.ang_a.long(), t.ang_b.long(), t.ang_c.long(), t.ang_t0.double(),
              t.ang_k.double())
    dih = _dihedral_tuple(t)
    thermo = (md.thermo_args, md.randoms.cpu().numpy())
    chi64 = torch.tensor(chi, dtype=torch.float64, device="cuda", requires_grad=True)
    args = (md, cfg, model, K, target.double(), n_bins, bonds, angles, dih, thermo)
    x0, v0 = md.r.double(), md.v.double()
    L64 = _torch_loss(x0, v0, chi64, *args)
    L64.backward()
    g64 = chi64.grad.cpu().numpy()
    assert float(loss.detach()) == pytest.approx(float(L64.detach()), rel=1e-4)
    pairs = [(i, j) for i in range(md.T) for j in range(i + 1, md.T) if chi[i, j] != 0]
    got = np.array([g[i, j] + g[j, i] for i, j in pairs])
    want = np.array([g64[i, j] + g64[j, i] for i, j in pairs])
    assert rel_rms(got, want) < 2e-3
    i, j = pairs[0]
    h = 1e-3
    with torch.no_grad():
        cp, cm = chi64.detach().clone(), chi64.detach().clone()
        cp[i, j] += h
        cp[j, i] += h
        cm[i, j] -= h
        cm[j, i] -= h
    fd = (float(_torch_loss(x0, v0, cp, *args).detach())
          - float(_torch_loss(x0, v0, cm, *args).detach())) / (2 * h)
    assert want[0] == pytest.approx(fd, rel=1e-5)
    md.check_errors()


def test_force_gradient_gap_shrinks_with_the_mesh():
    """||F + dW/dx|| / ||F|| (the MD force against the exact derivative of
    the discrete energy) on one configuration at three mesh spacings: it
    shrinks as the mesh is refined.  reference_gradient=True returns minus
    the MD force exactly."""
    from hymd_gb300 import adjoint, systems
    from hymd_gb300.field import ParticleMesh
    s = systems.lipid_membrane(seed=8, n_lipids=60, n_water=900, box=5.6, mesh=20)
    cfg = s["config"]
    names = cfg.unique_names
    T = cfg.n_types
    chi = np.zeros((T, T))
    for c in cfg.chi:
        i, j = names.index(c.atom_1), names.index(c.atom_2)
        chi[i, j] = chi[j, i] = c.interaction_energy
    pos = torch.tensor(s["positions"], dtype=torch.float32, device="cuda")
    typ = torch.tensor(s["types"], dtype=torch.int32, device="cuda")
    gaps = []
    for n in (14, 28, 56):
        pm = ParticleMesh([n, n, n], cfg.box(), T, device="cuda")
        gaps.append(adjoint.gradient_gap(pos, typ, pm, cfg.m, chi, cfg.kappa, cfg.sigma,
                                         cfg.rho0, cfg.a if cfg.a is not None else cfg.rho0))
    assert gaps[0] > gaps[1] > gaps[2], gaps
    x = pos.clone().requires_grad_(True)
    pm = ParticleMesh([28, 28, 28], cfg.box(), T, device="cuda")
    W = adjoint.field_energy(x, typ, pm, cfg.m, chi, cfg.kappa, cfg.sigma, cfg.rho0,
                             cfg.a if cfg.a is not None else cfg.rho0, reference_gradient=True)
    (g,) = torch.autograd.grad(W, x)
    from hymd_gb300 import _lib
    F = torch.empty_like(pos)
    _lib.call("hpf_field_step", pm._h, _lib.ptr(pos), _lib.ptr(typ), pos.shape[0],
              _lib.dvec(cfg.m), _lib.ptr(F), None, None, None, _lib.stream_ptr())
    assert torch.equal(g, -F)


def test_pic_force_vjp_matches_torch_autograd():
    """hpf_pic_force_vjp against the FP64 torch PIC force differentiated by
    autograd (the forward against hpf_pic_step first)."""
    from hymd_gb300 import _lib
    from hymd_gb300.reverse import ForceModel
    s, cfg, md, chi = _peptides(charged=True)
    model = ForceModel(md)
    q = s["charges"].astype(np.float64)
    assert np.count_nonzero(q) > 0
    F32 = torch.empty_like(md.r)
    _lib.call("hpf_pic_step", md.pm._h, _lib.ptr(md.r), _lib.ptr(md.charges), md.n,
              model.elec_factor, _lib.ptr(F32), None, None, None, None, None, None,
              _lib.stream_ptr())
    x = md.r.double().clone().requires_grad_(True)
    F = tf.pic_force(x, q, cfg.mesh(), list(cfg.box()), model.sigma, model.elec_factor)
    assert rel_rms(F32.cpu().numpy(), F.detach().cpu().numpy()) < 1e-5
    rng = np.random.default_rng(6)
    lam = torch.tensor(rng.normal(size=(md.n, 3)), dtype=torch.float32, device="cuda")
    g = torch.empty_like(md.r)
    _lib.call("hpf_pic_force_vjp", md.pm._h, _lib.ptr(md.r), _lib.ptr(md.charges), md.n,
              model.elec_factor, _lib.ptr(lam), _lib.ptr(g), _lib.stream_ptr())
    (lam.double() * F).sum().backward()
    assert rel_rms(g.cpu().numpy(), x.grad.cpu().numpy()) < 1e-4
    md.check_errors()


def test_profile_loss_gradient_with_charges_dihedrals_and_csvr():
    """The K-step chi gradient through a charged peptide trajectory (field +
    PIC_Spectral forces, CBT four-body terms, CSVR every outer step) against
    the FP64 torch trajectory, and that against a central finite difference."""
    from hymd_gb300.reverse import ForceModel, profile_loss
    s, cfg, md, chi = _peptides(charged=True)
    md.couple(thermostat=True, seed=8, n_steps=50)
    model = ForceModel(md)
    K, n_bins = 4, 20
    rng = np.random.default_rng(7)
    target = torch.tensor(rng.uniform(0.0, 3.0, size=(md.T, n_bins)), dtype=torch.float32,
                          device="cuda")
    chi_t = torch.tensor(chi, dtype=torch.float32, device="cuda", requires_grad=True)
    loss, _ = profile_loss(md.r.clone(), md.v.clone(), chi_t, model, K, target, n_bins=n_bins,
                           segment=2)
    loss.backward()
    g = chi_t.grad.double().cpu().numpy()
    t = md.topo
    bonds = (t.bond_a.long(), t.bond_b.long(), t.bond_r0.double(), t.bond_k.double())
    angles = (t.ang_a.long(), t.ang_b.long(), t.ang_c.long(), t.ang_t0.double(),
              t.ang_k.double())
    dih = _dihedral_tuple(t)
    thermo = (md.thermo_args, md.randoms.cpu().numpy())
    q = s["charges"].astype(np.float64)
    chi64 = torch.tensor(chi, dtype=torch.float64, device="cuda", requires_grad=True)
    args = (md, cfg, model, K, target.double(), n_bins, bonds, angles, dih, thermo, q)
    x0, v0 = md.r.double(), md.v.double()
    L64 = _torch_loss(x0, v0, chi64, *args)
    L64.backward()
    g64 = chi64.grad.cpu().numpy()
    assert float(loss.detach()) == pytest.approx(float(L64.detach()), rel=1e-4)
    pairs = [(i, j) for i in range(md.T) for j in range(i + 1, md.T) if chi[i, j] != 0]
    got = np.array([g[i, j] + g[j, i] for i, j in pairs])
    want = np.array([g64[i, j] + g64[j, i] for i, j in pairs])
    assert rel_rms(got, want) < 2e-3
    i, j = pairs[0]
    h = 1e-3
    with torch.no_grad():
        cp, cm = chi64.detach().clone(), chi64.detach().clone()
        cp[i, j] += h
        cp[j, i] += h
        cm[i, j] -= h
        cm[j, i] -= h
    fd = (float(_torch_loss(x0, v0, cp, *args).detach())
          - float(_torch_loss(x0, v0, cm, *args).detach())) / (2 * h)
    assert want[0] == pytest.approx(fd, rel=1e-5)
    md.check_errors()
