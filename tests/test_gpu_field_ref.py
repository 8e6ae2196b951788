"""The CUDA path against outputs of the reference's own code.

tests/golden/field_ref.npz holds what the unmodified hymd/field.py,
pressure.py, thermostat.py and barostat_scr.py computed (in FP64, through a
numpy stand-in for the pmesh library; tests/golden/make_field_ref.py).  Here
the drop-in entry points run the same inputs on the GPU.

Tolerances (the path's contract): per-particle forces within 1e-5 relative
RMS; energies and the pressure vector within 1e-6 relative (pressure: of its
largest field component); thermostat velocities within FP32 rounding (1e-6
relative) and box / positions after a barostat step within 1e-6; GPE
(an iterative FP32 solve): forces 1e-4 relative RMS, energy 1e-5, and the
same iteration count as the reference within one.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

FIX = np.load(os.path.join(os.path.dirname(__file__), "golden", "field_ref.npz"))
FORCE_RTOL = 1e-5
ENERGY_RTOL = 1e-6


def rel_rms(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def case(pre):
    d = {k[len(pre):]: FIX[k] for k in FIX.files if k.startswith(pre)}
    sigma, kappa, mass, rho0, a = d["scalars"]
    d.update(sigma=float(sigma), kappa=float(kappa), mass=float(mass), rho0=float(rho0),
             a=float(a))
    return d


def make_config(d, kind="DefaultWithChi", **extra):
    from hymd_gb300.config import Config
    from hymd_gb300.force import Chi
    T = len(d["m"])
    names = [chr(65 + t) for t in range(T)]
    chi = [Chi(names[i], names[j], float(d["chi"][i, j])) for i in range(T)
           for j in range(i + 1, T)]
    cfg = Config(n_steps=1, time_step=0.03, mesh_size=[int(x) for x in d["mesh"]],
                 sigma=d["sigma"], kappa=d["kappa"], box_size=np.array(d["box"]),
                 n_particles=len(d["positions"]), n_types=T, mass=d["mass"], hamiltonian=kind,
                 unique_names=names, type_to_name_map=dict(enumerate(names)), chi=chi,
                 m=[float(x) for x in d["m"]], respa_inner=10, tau=0.1,
                 target_temperature=323.0, type_charges=[0.0] * T)
    for k, v in extra.items():
        setattr(cfg, k, v)
    return cfg


def field_setup(d, cfg, positions=None):
    from hymd_gb300 import field as gf
    from hymd_gb300.hamiltonian import get_hamiltonian
    ham = get_hamiltonian(cfg)
    assert cfg.rho0 == pytest.approx(d["rho0"], rel=1e-12)
    pm, fl, ecl, cl = gf.initialize_pm(None, cfg)
    r = d["positions"] if positions is None else positions
    R = torch.as_tensor(np.asarray(r, np.float32), device="cuda")
    Ty = torch.as_tensor(d["types"].astype(np.int32), device="cuda")
    return gf, ham, pm, fl, ecl, cl, R, Ty


def check_pressure(P, Pref):
    scale = np.max(np.abs(Pref[:6]))
    assert np.max(np.abs(np.asarray(P) - Pref)) <= ENERGY_RTOL * scale, (P, Pref)


@pytest.mark.parametrize("name", ["chi3_cubic", "chi3_ragged", "nochi2", "sqphi2"])
def test_field_step_matches_reference(name):
    from hymd_gb300.pressure import comp_pressure
    d = case(f"field/{name}/")
    cfg = make_config(d, str(d["kind"]))
    gf, ham, pm, fl, _, _, R, Ty = field_setup(d, cfg)
    phi, phi_fourier, force_on_grid, v_ext_fourier, v_ext, phi_transfer, phi_lap = fl
    gf.update_field(phi, phi_lap, phi_transfer, None, force_on_grid, ham, pm, R, Ty, cfg, v_ext,
                    phi_fourier, v_ext_fourier, cfg.m, compute_potential=True)
    F = torch.zeros_like(R)
    gf.compute_field_force(None, R, force_on_grid, F, Ty, cfg.n_types)
    assert rel_rms(F.cpu().numpy(), d["forces"]) < FORCE_RTOL
    if "phi" in d:
        for t in range(cfg.n_types):
            assert rel_rms(phi[t].cpu().numpy(), d["phi"][t]) < 1e-6
            assert rel_rms(v_ext[t].cpu().numpy(), d["v_ext"][t]) < FORCE_RTOL
    vel = torch.as_tensor(d["velocities"], device="cuda")
    W, KE, Wq = gf.compute_field_and_kinetic_energy(phi, None, None, vel, ham, R, Ty, v_ext, cfg,
                                                    None)
    assert W == pytest.approx(d["energies"][0], rel=ENERGY_RTOL)
    assert KE == pytest.approx(d["energies"][1], rel=ENERGY_RTOL)
    P = comp_pressure(phi, None, None, ham, vel, cfg, phi_fourier, phi_lap, phi_transfer, R,
                      d["bond_pr"], d["angle_pr"])
    check_pressure(P, d["pressure"])
    pm.check_errors()


def test_pic_matches_reference():
    from hymd_gb300.pressure import comp_pressure
    d = case("pic/")
    cfg = make_config(d, coulombtype="PIC_Spectral", dielectric_const=float(d["dielectric_const"]),
                      type_charges=[float(x) for x in d["type_charges"]])
    gf, ham, pm, fl, ecl, cl, R, Ty = field_setup(d, cfg)
    Q = torch.as_tensor(d["charges"].astype(np.float32), device="cuda")
    cfg.self_energy = gf.compute_self_energy_q(cfg, Q)
    assert cfg.self_energy == pytest.approx(float(d["self_energy"]), rel=ENERGY_RTOL)
    phi, phi_fourier, force_on_grid, v_ext_fourier, v_ext, phi_transfer, phi_lap = fl
    phi_q, phi_q_fourier, psi, elec_field = ecl
    elec_field_fourier, psi_fourier = cl
    gf.update_field(phi, phi_lap, phi_transfer, None, force_on_grid, ham, pm, R, Ty, cfg, v_ext,
                    phi_fourier, v_ext_fourier, cfg.m, compute_potential=True)
    F = torch.zeros_like(R)
    gf.compute_field_force(None, R, force_on_grid, F, Ty, cfg.n_types)
    Fq = torch.zeros_like(R)
    gf.update_field_force_q(Q, phi_q, phi_q_fourier, psi, psi_fourier, elec_field_fourier,
                            elec_field, Fq, None, ham, pm, R, cfg)
    assert rel_rms(F.cpu().numpy(), d["forces"]) < FORCE_RTOL
    assert rel_rms(Fq.cpu().numpy(), d["elec_forces"]) < FORCE_RTOL
    assert rel_rms(psi.cpu().numpy(), d["psi"]) < FORCE_RTOL
    vel = torch.as_tensor(d["velocities"], device="cuda")
    W, KE, Wq = gf.compute_field_and_kinetic_energy(phi, phi_q, psi, vel, ham, R, Ty, v_ext, cfg,
                                                    None)
    assert W == pytest.approx(d["energies"][0], rel=ENERGY_RTOL)
    assert Wq == pytest.approx(d["energies"][2], rel=ENERGY_RTOL)
    P = comp_pressure(phi, phi_q, psi, ham, vel, cfg, phi_fourier, phi_lap, phi_transfer, R,
                      d["bond_pr"], d["angle_pr"])
    check_pressure(P, d["pressure"])
    pm.check_errors()


def test_gpe_two_calls_match_reference():
    d = case("gpe/")
    T = len(d["m"])
    cfg = make_config(d, coulombtype="PIC_Spectral_GPE",
                      type_charges=[float(x) for x in d["type_charges"]],
                      dielectric_type=[float(x) for x in d["dielectric_type"]],
                      conv_crit=float(d["conv"][0]), pol_mixing=float(d["conv"][1]),
                      convergence_type="max_diff")
    gf, ham, pm, fl, ecl, cl, R, Ty = field_setup(d, cfg)
    phi, phi_fourier, force_on_grid, v_ext_fourier, v_ext, phi_transfer, phi_lap = fl
    phi_q, phi_q_fourier, psi, elec_field = ecl
    (phi_eps, phi_eps_fourier, phi_eta, phi_eta_fourier, phi_pol, phi_pol_prev, elec_dot,
     elec_field_contrib, Vbar_elec, Vbar_elec_fourier, force_mesh_elec,
     force_mesh_elec_fourier) = cl
    Q = torch.as_tensor(d["charges"].astype(np.float32), device="cuda")
    for call, key in enumerate(("positions", "positions2")):
        R = torch.as_tensor(d[key], device="cuda")
        gf.update_field(phi, phi_lap, phi_transfer, None, force_on_grid, ham, pm, R, Ty, cfg,
                        v_ext, phi_fourier, v_ext_fourier, cfg.m)
        F = torch.zeros_like(R)
        Vb, eps_g, dot = gf.update_field_force_q_GPE(
            None, phi, Ty, Q, phi_q, phi_q_fourier, phi_eps, phi_eps_fourier, phi_eta,
            phi_eta_fourier, phi_pol_prev, phi_pol, elec_field, F, elec_field_contrib, psi,
            Vbar_elec, Vbar_elec_fourier, force_mesh_elec, force_mesh_elec_fourier, ham, None,
            None, pm, R, cfg)
        W = gf.compute_field_energy_q_GPE(cfg, eps_g, None, dot)
        torch.cuda.synchronize()
        c = f"call{call}/"
        assert abs(pm.gpe_iterations - int(d[c + "iterations"])) <= 1, (call, pm.gpe_iterations)
        assert rel_rms(eps_g.cpu().numpy(), d[c + "phi_eps"]) < 1e-6
        assert rel_rms(F.cpu().numpy(), d[c + "elec_forces"]) < 1e-4
        assert rel_rms(psi.cpu().numpy(), d[c + "psi"]) < 1e-4
        assert W == pytest.approx(float(d[c + "energy"]), rel=1e-5)
    assert not torch.any(phi_pol_prev) and not torch.any(phi_pol)
    pm.check_errors()


@pytest.mark.parametrize("name", ["one_com", "one_nocom", "two_com", "two_nocom"])
def test_csvr_matches_reference(name):
    """Device CSVR (hpf_csvr) on the reference's velocities and draws: one and
    two coupling groups, with and without centre-of-mass removal (without it,
    each group's rescaling uses the whole system's current kinetic energy and
    scales every particle, as thermostat.py:190-219 does)."""
    from hymd_gb300 import _lib
    d = {k.split("/")[-1]: FIX[k] for k in FIX.files if k.startswith(f"csvr/{name}/")}
    mass, gas, temp, dt_o, tau = (float(x) for x in d["params"])
    group = d["group"].astype(np.int32)
    ng = int(group.max()) + 1
    v = torch.as_tensor(d["v0"].astype(np.float32), device="cuda")
    G = torch.as_tensor(group, device="cuda")
    draws = np.zeros(4)
    draws[: 2 * ng] = d["draws"]
    table = torch.as_tensor(draws, device="cuda")
    a = _lib.CsvrArgs()
    a.n_groups, a.remove_com, a.n_steps, a.stride = ng, int(name.endswith("_com")), 1, 4
    a.offset, a.advance, a.every = 0, 1, 1
    for g in range(ng):
        a.count[g] = float(np.sum(group == g))
    a.mass, a.gas_constant, a.target_temperature = mass, gas, temp
    a.c = float(np.exp(-dt_o / tau))
    counter = torch.zeros(4, dtype=torch.int32, device="cuda")
    state = torch.zeros(16, dtype=torch.float64, device="cuda")
    ws = _lib.new_workspace(v.device)
    err = torch.zeros(8, dtype=torch.int32, device="cuda")
    _lib.call("hpf_csvr", _lib.ptr(v), _lib.ptr(G), v.shape[0], None, 0, 0.0,
              _lib.ctypes.byref(a), _lib.ptr(table), _lib.ptr(counter), _lib.ptr(state),
              _lib.ptr(ws), _lib.ptr(err), _lib.stream_ptr())
    got = v.cpu().numpy()
    want = d["v1"]
    assert np.max(np.abs(got - want)) <= 1e-6 * np.max(np.abs(want))
    work = float(state[8].item() + state[9].item())
    assert work == pytest.approx(float(d["work"]), rel=1e-5)
    assert int(counter[0].item()) == 1
    assert not torch.any(err)


@pytest.mark.parametrize("mode", ["iso", "semi", "semi_lateral"])
def test_scr_matches_reference(mode):
    """Device SCR step (hpf_scr_isotropic) after a field evaluation at the
    reference's positions, with its bond/angle virials and draws: pressure,
    box and positions against barostat_scr.py's result."""
    from hymd_gb300 import _lib
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    d = case(f"scr/{mode}/")
    tau_p, n_b, dt_o, temp, gas = (float(x) for x in d["params"])
    cfg = make_config(d, barostat="isotropic" if mode == "iso" else "semiisotropic",
                      tau_p=tau_p, n_b=int(n_b), rho0=d["rho0"], a=d["a"])
    ham = get_hamiltonian(cfg)
    md = RespaMD(d["positions"], d["velocities"], d["types"], cfg, ham)
    targets = d["targets"]
    md.couple(thermostat=False, barostat="isotropic" if mode == "iso" else "semiisotropic",
              seed=0, n_steps=1,
              target_pressure=float(targets[0]) if mode == "iso" else tuple(targets))
    table = np.zeros(md.randoms.numel())
    table[: (1 if mode == "iso" else 2)] = d["draws"][: (1 if mode == "iso" else 2)]
    md.randoms.copy_(torch.as_tensor(table))
    st = _lib.stream_ptr()
    md._field(st, md.field_sums)
    md.bonded_out.zero_()
    md.bonded_out[1:4] = torch.as_tensor(d["bond_pr"])
    md.bonded_out[5:8] = torch.as_tensor(d["angle_pr"])
    md._barostat(st)  # pressure, scale factors, box, then the position update
    torch.cuda.synchronize()
    P = d["pressure"]
    state = md.state.cpu().numpy()
    if mode == "iso":
        assert state[13] == pytest.approx(np.average(P[-3:-1]) * 16.61, rel=1e-5)
    else:
        assert state[13] == pytest.approx((P[-3] + P[-2]) / 2 * 16.61, rel=1e-5)
        assert state[15] == pytest.approx(P[-1] * 16.61, rel=1e-5)
    box = md.box_now()
    assert np.allclose(box, d["box_after"], rtol=1e-6)
    assert np.allclose(md.r.cpu().numpy(), d["positions_after"], rtol=1e-6, atol=1e-6)
    md.check_errors()
