"""PIC_Spectral_GPE electrostatics (hpf_gpe_step through the drop-in
update_field_force_q_GPE) against the FP64 oracle restatement of
hymd/field.py:706-1112.

Two consecutive calls with the max_diff and csum convergence measures; each
starts the polarisation iteration from the caller's unchanged phi_pol_prev,
as the reference does (it rebinds the name locally, field.py:1010-1024).  Tolerances: dielectric grid 1e-6 relative, forces 1e-4 relative
RMS (FP32 transforms through the iterative solve), energy 1e-5 relative;
iteration counts within 2.  (Systems with empty regions, where the total
filtered density falls below 1e-6, are not tested: there the reference keeps
a zero dielectric and its iteration diverges.)
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import field as of  # noqa: E402
from oracle import hamiltonian as oh  # noqa: E402


def rel_rms(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def _system(conv, seed=21, mesh=(24, 24, 26)):
    from hymd_gb300.config import Config
    from hymd_gb300.force import Chi
    rng = np.random.default_rng(seed)
    T, n = 3, 3000
    box = np.array([5.0, 5.0, 5.5])
    r = rng.uniform(0, 1, (n, 3)) * box
    r[: n // 3] = np.mod(box / 2 + rng.normal(0, 0.6, (n // 3, 3)), box)
    r = r.astype(np.float32)
    types = rng.integers(0, T, n).astype(np.int32)
    q = np.zeros(n, np.float32)
    k = rng.permutation(n)[: n // 5]
    q[k] = rng.choice([-1.0, 1.0], len(k)).astype(np.float32)
    names = ["A", "B", "C"]
    chi = [Chi("A", "B", 12.0), Chi("A", "C", 4.0), Chi("B", "C", 20.0)]
    cfg = Config(n_steps=1, time_step=0.03, mesh_size=list(mesh), sigma=0.5,
                 kappa=0.05, box_size=box, n_particles=n, n_types=T, mass=72.0,
                 hamiltonian="DefaultWithChi", unique_names=names,
                 type_to_name_map=dict(enumerate(names)), chi=chi, m=[1.0, 1.0, 1.0],
                 coulombtype="PIC_Spectral_GPE", type_charges=[0.3, -0.3, 0.0],
                 dielectric_type=[80.0, 2.0, 10.0],
                 conv_crit=1e-7 if conv == "max_diff" else 1e-4, pol_mixing=0.6,
                 convergence_type=conv)
    return cfg, r, types, q


@pytest.mark.parametrize("conv,mesh", [("max_diff", (24, 24, 26)), ("csum", (24, 24, 26)),
                                       ("max_diff", (24, 24, 24)), ("csum", (32, 32, 32))])
def test_gpe_matches_oracle(conv, mesh):
    """24 x 24 x 26 takes the cuFFT transforms; the cubic meshes the fused
    spectral passes (the polarisation loop and the final psi, E on the PIC
    chain's passes without the filter)."""
    from hymd_gb300 import field as gf
    from hymd_gb300.hamiltonian import get_hamiltonian
    cfg, r, types, q = _system(conv, mesh=mesh)
    T = cfg.n_types
    ham = get_hamiltonian(cfg)
    pm, fl, ecl, cl = gf.initialize_pm(None, cfg)
    phi, phi_fourier, force_on_grid, v_ext_fourier, v_ext, phi_transfer, phi_lap = fl
    phi_q, phi_q_fourier, psi, elec_field = ecl
    (phi_eps, phi_eps_fourier, phi_eta, phi_eta_fourier, phi_pol, phi_pol_prev, elec_dot,
     elec_field_contrib, Vbar_elec, Vbar_elec_fourier, force_mesh_elec,
     force_mesh_elec_fourier) = cl
    R = torch.as_tensor(r, device="cuda")
    Ty = torch.as_tensor(types, device="cuda")
    Q = torch.as_tensor(q, device="cuda")
    assert pm.spectral == ("cufft" if mesh[2] == 26 else "fused")
    gf.update_field(phi, phi_lap, phi_transfer, None, force_on_grid, ham, pm, R, Ty, cfg, v_ext,
                    phi_fourier, v_ext_fourier, cfg.m)
    names = cfg.unique_names
    chim = np.zeros((T, T))
    for c in cfg.chi:
        i, j = names.index(c.atom_1), names.index(c.atom_2)
        chim[i, j] = chim[j, i] = c.interaction_energy
    fun = oh.quadratic_from_params("DefaultWithChi", T, cfg.kappa, cfg.rho0, cfg.a, chim)
    ref_field = of.update_field(r.astype(np.float64), types, T, cfg.mesh(), cfg.box(), cfg.m,
                                fun, cfg.sigma)
    nshape = tuple(cfg.mesh())
    state = dict(phi_eps=np.zeros(nshape), pol_prev=np.zeros(nshape), contrib=np.zeros(nshape))
    F = torch.zeros_like(R)
    for call in range(2):
        Vb, eps_g, dot = gf.update_field_force_q_GPE(
            None, phi, Ty, Q, phi_q, phi_q_fourier, phi_eps, phi_eps_fourier, phi_eta,
            phi_eta_fourier, phi_pol_prev, phi_pol, elec_field, F, elec_field_contrib, psi,
            Vbar_elec, Vbar_elec_fourier, force_mesh_elec, force_mesh_elec_fourier, ham, None,
            None, pm, R, cfg)
        W = gf.compute_field_energy_q_GPE(cfg, eps_g, None, dot)
        ref = of.gpe_step(ref_field["phi"], q, r, types, T, cfg.mesh(), cfg.box(), cfg.sigma,
                          cfg.dielectric_type, cfg.type_charges, state, conv_crit=cfg.conv_crit,
                          mixing=cfg.pol_mixing, conv_kind=conv)
        torch.cuda.synchronize()
        assert abs(pm.gpe_iterations - ref["iterations"]) <= 2, (call, pm.gpe_iterations,
                                                                ref["iterations"])
        assert rel_rms(phi_eps.cpu().numpy(), ref["phi_eps"]) < 1e-6
        assert rel_rms(psi.cpu().numpy(), ref["psi"]) < 1e-4
        assert rel_rms(F.cpu().numpy(), ref["forces"]) < 1e-4, call
        assert W == pytest.approx(ref["energy"], rel=1e-5)
        assert rel_rms(Vb[0].cpu().numpy(), ref["Vbar"][0]) < 1e-4
    assert not torch.any(phi_pol_prev) and not torch.any(phi_pol)  # caller's grids untouched
    pm.check_errors()


def test_gpe_loop_graph_follows_parameters():
    """The polarisation loop runs as a cached CUDA graph with a device-side
    loop test: calls on one mesh context with another tolerance, or with
    max_iter = 0 (no iteration), rebuild it, and each call's iteration count
    and forces follow the FP64 oracle with that tolerance."""
    from hymd_gb300 import _lib, field as gf
    from hymd_gb300.hamiltonian import get_hamiltonian
    cfg, r, types, q = _system("max_diff", seed=23, mesh=(24, 24, 24))
    T = cfg.n_types
    ham = get_hamiltonian(cfg)
    pm, fl, ecl, cl = gf.initialize_pm(None, cfg)
    phi, phi_fourier, force_on_grid, v_ext_fourier, v_ext, phi_transfer, phi_lap = fl
    phi_q, phi_q_fourier, psi, elec_field = ecl
    (phi_eps, phi_eps_fourier, phi_eta, phi_eta_fourier, phi_pol, phi_pol_prev, elec_dot,
     elec_field_contrib, Vbar_elec, Vbar_elec_fourier, force_mesh_elec,
     force_mesh_elec_fourier) = cl
    R = torch.as_tensor(r, device="cuda")
    Ty = torch.as_tensor(types, device="cuda")
    Q = torch.as_tensor(q, device="cuda")
    gf.update_field(phi, phi_lap, phi_transfer, None, force_on_grid, ham, pm, R, Ty, cfg, v_ext,
                    phi_fourier, v_ext_fourier, cfg.m)
    names = cfg.unique_names
    chim = np.zeros((T, T))
    for c in cfg.chi:
        i, j = names.index(c.atom_1), names.index(c.atom_2)
        chim[i, j] = chim[j, i] = c.interaction_energy
    fun = oh.quadratic_from_params("DefaultWithChi", T, cfg.kappa, cfg.rho0, cfg.a, chim)
    ref_field = of.update_field(r.astype(np.float64), types, T, cfg.mesh(), cfg.box(), cfg.m,
                                fun, cfg.sigma)
    nshape = tuple(cfg.mesh())
    state = dict(phi_eps=np.zeros(nshape), pol_prev=np.zeros(nshape), contrib=np.zeros(nshape))
    F = torch.zeros_like(R)
    counts = []
    for crit in (1e-3, 1e-7, 1e-3):
        cfg.conv_crit = crit
        gf.update_field_force_q_GPE(
            None, phi, Ty, Q, phi_q, phi_q_fourier, phi_eps, phi_eps_fourier, phi_eta,
            phi_eta_fourier, phi_pol_prev, phi_pol, elec_field, F, elec_field_contrib, psi,
            Vbar_elec, Vbar_elec_fourier, force_mesh_elec, force_mesh_elec_fourier, ham, None,
            None, pm, R, cfg)
        ref = of.gpe_step(ref_field["phi"], q, r, types, T, cfg.mesh(), cfg.box(), cfg.sigma,
                          cfg.dielectric_type, cfg.type_charges, state, conv_crit=crit,
                          mixing=cfg.pol_mixing, conv_kind="max_diff")
        torch.cuda.synchronize()
        assert abs(pm.gpe_iterations - ref["iterations"]) <= 2, (crit, pm.gpe_iterations,
                                                                ref["iterations"])
        assert rel_rms(F.cpu().numpy(), ref["forces"]) < 1e-4, crit
        counts.append(pm.gpe_iterations)
    assert counts[0] < counts[1] and counts[0] == counts[2]
    # max_iter = 0 through the C entry: the loop body never runs
    eps = _lib.dvec(cfg.dielectric_type)
    qt = _lib.dvec(cfg.type_charges)
    phi_all = torch.stack([p for p in phi]) if isinstance(phi, (list, tuple)) else phi
    pol = torch.zeros(nshape, dtype=torch.float32, device="cuda")
    it = _lib.ctypes.c_int(-1)
    _lib.call("hpf_gpe_step", pm._h, _lib.ptr(R), _lib.ptr(Ty), _lib.ptr(Q), R.shape[0],
              _lib.ptr(phi_all.contiguous()), eps, qt, float(cfg.coulomb_constant), 1e-7, 0.6, 0,
              0, _lib.ptr(phi_eps), _lib.ptr(pol), _lib.ptr(elec_field_contrib), _lib.ptr(F),
              None, None, None, None, None, _lib.ctypes.byref(it), _lib.stream_ptr())
    assert it.value == 0 and not torch.any(pol)
    pm.check_errors()
