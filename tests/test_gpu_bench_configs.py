"""Parity at the benchmark configurations, full size: the 10k-bead melt
(mesh 32^3), the 162k-bead membrane (64^3, 5 types) and the 500k-bead charged
peptides (128^3, PIC_Spectral, cosine + combined bending-torsion dihedrals);
and the same peptides under PIC_Spectral_GPE (the bench's GPE workload).

For each: one field evaluation through the drop-in API (update_field,
compute_field_force, compute_field_and_kinetic_energy, comp_pressure; with
charges also update_field_force_q) and the bonded forces of the fused rRESPA
plan (hpf_respa_forces), against the FP64 oracle (itself pinned to the
reference's own field.py / pressure.py by tests/golden/field_ref.npz) and the
real(8) C restatement of the Fortran bonded kernels.

Tolerances (the path's contract): forces within 1e-5 relative RMS, field and
electrostatic energies within 1e-6 relative, the pressure vector within 1e-6
of its largest field component.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5
ENERGY_RTOL = 1e-6


def rel_rms(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


@pytest.mark.parametrize("workload", ["melt10k", "membrane162k", "peptide500k"])
def test_full_size_field_and_bonded_match_oracle(workload):
    from hymd_gb300 import _lib, systems
    from hymd_gb300 import field as gf
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    from hymd_gb300.pressure import comp_pressure
    from oracle import bonded as ob
    from oracle import field as of
    from oracle import hamiltonian as oh

    of.FFT_WORKERS = os.cpu_count() or 1
    s = systems.BUILDERS[workload](seed=2)
    cfg = s["config"]
    T = cfg.n_types
    ham = get_hamiltonian(cfg)
    R = torch.as_tensor(s["positions"], device="cuda")
    V = torch.as_tensor(s["velocities"], device="cuda")
    Ty = torch.as_tensor(s["types"], device="cuda")
    pm, fl, ecl, cl = gf.initialize_pm(None, cfg)
    phi, phi_fourier, force_on_grid, v_ext_fourier, v_ext, phi_transfer, phi_lap = fl
    gf.update_field(phi, phi_lap, phi_transfer, None, force_on_grid, ham, pm, R, Ty, cfg, v_ext,
                    phi_fourier, v_ext_fourier, cfg.m)
    F = torch.zeros_like(R)
    gf.compute_field_force(None, R, force_on_grid, F, Ty, T)
    charged = s.get("charges") is not None and cfg.coulombtype == "PIC_Spectral"
    psi = phi_q = None
    if charged:
        Q = torch.as_tensor(s["charges"], device="cuda")
        cfg.self_energy = gf.compute_self_energy_q(cfg, Q)
        phi_q, phi_q_fourier, psi, elec_field = ecl
        elec_field_fourier, psi_fourier = cl
        Fq = torch.zeros_like(R)
        gf.update_field_force_q(Q, phi_q, phi_q_fourier, psi, psi_fourier, elec_field_fourier,
                                elec_field, Fq, None, ham, pm, R, cfg)
    W, KE, Wq = gf.compute_field_and_kinetic_energy(phi, phi_q, psi, V, ham, R, Ty, v_ext, cfg,
                                                    None)
    bond_pr = np.array([120.0, -40.0, 75.0])
    angle_pr = np.array([-30.0, 12.0, 8.0])
    P = comp_pressure(phi, phi_q, psi, ham, V, cfg, phi_fourier, phi_lap, phi_transfer, R,
                      bond_pr, angle_pr)

    r64 = s["positions"].astype(np.float64)
    fun = oh.functional_of_config(cfg)
    ref = of.update_field(r64, s["types"], T, cfg.mesh(), cfg.box(), cfg.m, fun, cfg.sigma)
    Fref = of.compute_field_force(ref["force_mesh"], r64, s["types"], T, cfg.mesh(), cfg.box())
    assert rel_rms(F.cpu().numpy(), Fref) < FORCE_RTOL
    Wref = of.field_energy(ref["phi"], fun, cfg.mesh(), cfg.box())
    assert W == pytest.approx(Wref, rel=ENERGY_RTOL)
    assert KE == pytest.approx(of.kinetic_energy(s["velocities"], cfg.mass), rel=ENERGY_RTOL)
    kw = {}
    if charged:
        qr = of.update_field_force_q(s["charges"].astype(np.float64), r64, cfg.mesh(), cfg.box(),
                                     cfg.sigma, cfg.dielectric_const)
        assert rel_rms(Fq.cpu().numpy(), qr["forces"]) < FORCE_RTOL
        Es = of.self_energy_q(s["charges"], cfg.sigma, cfg.dielectric_const)
        assert cfg.self_energy == pytest.approx(Es, rel=ENERGY_RTOL)
        Wq_ref = of.field_q_energy(qr["phi_q"], qr["psi"], Es, cfg.mesh(), cfg.box())
        assert Wq == pytest.approx(Wq_ref, rel=ENERGY_RTOL)
        kw = dict(phi_q=qr["phi_q"], psi=qr["psi"], self_energy=Es,
                  type_charges=list(cfg.type_charges))
    Pref = of.comp_pressure(ref["phi"], ref["phi_fourier"], fun, s["velocities"], cfg.mass,
                            cfg.mesh(), cfg.box(), cfg.sigma, bond_pr, angle_pr, **kw)
    assert np.max(np.abs(P - Pref)) <= ENERGY_RTOL * np.max(np.abs(Pref[:6]))
    pm.check_errors()

    # bonded forces of the fused plan against the real(8) restatement.  The
    # recipes build chains with bonds at exactly r0, where the bond forces are
    # FP32 rounding noise; a seeded 0.02 nm jitter gives them a scale.
    rng = np.random.default_rng(11)
    rj = np.mod(s["positions"] + rng.normal(0, 0.02, s["positions"].shape),
                cfg.box()).astype(np.float32)
    r64 = rj.astype(np.float64)
    md = RespaMD(rj, s["velocities"], s["types"], cfg, ham, topology=s["topology"],
                 max_block_beads=24)
    fb = torch.zeros_like(md.r)
    _lib.call("hpf_respa_forces", md.plan, _lib.ptr(md.r), _lib.ptr(fb), _lib.ptr(md.box), None,
              _lib.ptr(md.err), _lib.stream_ptr())
    torch.cuda.synchronize()
    md.check_errors()
    (b2a, b2b, b2r, b2k, b3a, b3b, b3c, b3t, b3k, b4a, b4b, b4c, b4d, b4coeff, b4type,
     b4last) = s["topology"]
    box = cfg.box()
    want = np.zeros_like(r64)
    if len(b2a):
        f = np.zeros_like(r64)
        ob.compute_bond_forces(f, r64, box, b2a, b2b, b2r, b2k, precision="double")
        want += f
    if len(b3a):
        f = np.zeros_like(r64)
        ob.compute_angle_forces(f, r64, box, b3a, b3b, b3c, b3t, b3k, precision="double")
        want += f
    if len(b4a):
        nd = len(b4a)
        f = np.zeros_like(r64)
        ob.compute_dihedral_forces(f, r64, np.zeros((nd, 4, 3)), np.zeros((nd, 6, 3, 3)), box,
                                   b4a, b4b, b4c, b4d, b4coeff, b4type, b4last, 0,
                                   precision="double")
        want += f
    sel = np.zeros(len(r64), bool)
    for idx in (b2a, b2b, b3a, b3b, b3c, b4a, b4b, b4c, b4d):
        sel[np.asarray(idx, np.int64)] = True
    assert rel_rms(fb.cpu().numpy()[sel], want[sel]) < FORCE_RTOL


def test_full_size_gpe_matches_oracle():
    """PIC_Spectral_GPE at the benchmark size: the 500k-bead charged peptides
    on 128^3 (the fused spectral passes and the loop graph), dielectric
    2 / 10 / 80 for BB / SC / W, max_diff to 1e-6, against the FP64 oracle's
    solve of the same inputs: the same iteration count, forces within 1e-5
    relative RMS (FP32 transforms through the iterative solve), energy within
    1e-5."""
    from hymd_gb300 import field as gf, systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from oracle import field as of
    from oracle import hamiltonian as oh
    s = systems.charged_peptides(seed=2)
    cfg = s["config"]
    cfg.coulombtype = "PIC_Spectral_GPE"
    cfg.dielectric_type = [2.0, 10.0, 80.0]
    cfg.conv_crit, cfg.pol_mixing, cfg.convergence_type = 1e-6, 0.6, "max_diff"
    T = cfg.n_types
    ham = get_hamiltonian(cfg)
    pm, fl, ecl, cl = gf.initialize_pm(None, cfg)
    assert pm.spectral == "fused"
    phi, phi_fourier, force_on_grid, v_ext_fourier, v_ext, phi_transfer, phi_lap = fl
    phi_q, phi_q_fourier, psi, elec_field = ecl
    (phi_eps, phi_eps_fourier, phi_eta, phi_eta_fourier, phi_pol, phi_pol_prev, elec_dot,
     elec_field_contrib, Vbar_elec, Vbar_elec_fourier, force_mesh_elec,
     force_mesh_elec_fourier) = cl
    R = torch.as_tensor(s["positions"], device="cuda")
    Ty = torch.as_tensor(s["types"], device="cuda")
    Q = torch.as_tensor(s["charges"], device="cuda")
    gf.update_field(phi, phi_lap, phi_transfer, None, force_on_grid, ham, pm, R, Ty, cfg, v_ext,
                    phi_fourier, v_ext_fourier, cfg.m)
    F = torch.zeros_like(R)
    _, eps_g, dot = gf.update_field_force_q_GPE(
        None, phi, Ty, Q, phi_q, phi_q_fourier, phi_eps, phi_eps_fourier, phi_eta,
        phi_eta_fourier, phi_pol_prev, phi_pol, elec_field, F, elec_field_contrib, psi,
        Vbar_elec, Vbar_elec_fourier, force_mesh_elec, force_mesh_elec_fourier, ham, None, None,
        pm, R, cfg)
    W = gf.compute_field_energy_q_GPE(cfg, eps_g, None, dot)
    names = cfg.unique_names
    chim = np.zeros((T, T))
    for c in cfg.chi:
        i, j = names.index(c.atom_1), names.index(c.atom_2)
        chim[i, j] = chim[j, i] = c.interaction_energy
    fun = oh.quadratic_from_params("DefaultWithChi", T, cfg.kappa, cfg.rho0, cfg.a, chim)
    ref_field = of.update_field(s["positions"].astype(np.float64), s["types"], T, cfg.mesh(),
                                cfg.box(), cfg.m, fun, cfg.sigma)
    nshape = tuple(cfg.mesh())
    state = dict(phi_eps=np.zeros(nshape), pol_prev=np.zeros(nshape), contrib=np.zeros(nshape))
    ref = of.gpe_step(ref_field["phi"], s["charges"], s["positions"], s["types"], T, cfg.mesh(),
                      cfg.box(), cfg.sigma, cfg.dielectric_type, [0.0] * T, state,
                      conv_crit=cfg.conv_crit, mixing=cfg.pol_mixing, conv_kind="max_diff")
    torch.cuda.synchronize()
    assert pm.gpe_iterations == ref["iterations"]
    assert rel_rms(F.cpu().numpy(), ref["forces"]) < FORCE_RTOL
    assert W == pytest.approx(ref["energy"], rel=1e-5)
    pm.check_errors()
