"""Device CSVR thermostat and SCR barostat against host restatements of
hymd/thermostat.py:111-219 and hymd/barostat_scr.py:34-284."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import field as of  # noqa: E402
from oracle import hamiltonian as oh  # noqa: E402


def _system():
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    s = systems.lipid_membrane(seed=4, n_lipids=200, n_water=3000, box=8.0, mesh=24)
    cfg = s["config"]
    cfg.tau_p = 1.0
    cfg.n_b = 1
    ham = get_hamiltonian(cfg)
    return s, cfg, ham


def _functional(cfg):
    T = cfg.n_types
    names = cfg.unique_names
    chi = np.zeros((T, T))
    for c in cfg.chi:
        i, j = names.index(c.atom_1), names.index(c.atom_2)
        chi[i, j] = chi[j, i] = c.interaction_energy
    return oh.quadratic_from_params("DefaultWithChi", T, cfg.kappa, cfg.rho0, cfg.a, chi)


def test_csvr_thermostat_matches_reference_formula():
    from hymd_gb300 import _lib
    from hymd_gb300.md import RespaMD
    s, cfg, ham = _system()
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    md.couple(thermostat=True, barostat=None, seed=3, n_steps=10)
    v0 = md.v.cpu().numpy().astype(np.float64)
    st = _lib.stream_ptr()
    md._thermostat(st)
    v1 = md.v.cpu().numpy()
    # host restatement with the same random numbers
    table = md.randoms.cpu().numpy().reshape(10, -1)
    R, S = table[0, 1], table[0, 2]
    N = len(v0)
    com = v0.sum(0) / N
    K = 0.5 * cfg.mass * np.sum((v0 - com) ** 2)
    Kt = 1.5 * cfg.gas_constant * N * cfg.target_temperature
    c = np.exp(-cfg.respa_inner * cfg.time_step / cfg.tau)
    a2 = c + (1 - c) * (S + R * R) * Kt / (3 * N * K) + 2 * R * np.sqrt(c * (1 - c) * Kt / (3 * N * K))
    vref = (v0 - com) * np.sqrt(a2) + com
    assert np.allclose(v1, vref, rtol=1e-5, atol=1e-6)
    assert int(md.counter[0].item()) == 1


def test_scr_barostat_matches_reference_formula():
    from hymd_gb300 import _lib
    from hymd_gb300.md import RespaMD
    s, cfg, ham = _system()
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    md.FUSE_PAINT = False  # the separate paint scales the positions (pos_scale below)
    md.couple(thermostat=False, barostat="isotropic", seed=5, n_steps=10)
    md.prime()
    r_field = md.r.cpu().numpy().copy()  # positions of the last field evaluation
    box0 = md.box_now()
    st = _lib.stream_ptr()
    md._inner_fused(st)  # inner loop; its last block runs the barostat on the box
    r_before = md.r.cpu().numpy().astype(np.float64)
    v = md.v.cpu().numpy()
    bonded = md.bonded_out.cpu().numpy()
    box1 = md.box_now()
    md._field(st, md.field_sums, pos_scale=md.state.data_ptr() + 12 * 8)  # rescales positions
    r_after = md.r.cpu().numpy()
    # host pressure: FP64 oracle field at r_field, bonded virials, kinetic energy
    fun = _functional(cfg)
    ref = of.update_field(r_field.astype(np.float64), s["types"], cfg.n_types, cfg.mesh(), box0,
                          cfg.m, fun, cfg.sigma)
    P18 = of.comp_pressure(ref["phi"], ref["phi_fourier"], fun, v, cfg.mass, cfg.mesh(), box0,
                           cfg.sigma, bonded[1:4], bonded[5:8])
    P = np.average(P18[-3:-1]) * 16.61
    R = md.randoms.cpu().numpy().reshape(10, -1)[0, 0]
    V = np.prod(box0)
    dt_o = cfg.respa_inner * cfg.time_step
    beta = 7.6e-4
    noise = np.sqrt(2.0 * 1 * cfg.gas_constant * cfg.target_temperature * beta * dt_o * 1
                    / (V * cfg.tau_p)) * R
    log_alpha = -1 * dt_o * beta / cfg.tau_p * (1.0 - P) + noise
    alpha = np.exp(log_alpha / 3.0)
    assert float(md.state[13].item()) == pytest.approx(P, rel=1e-5, abs=5e-2)
    assert float(md.bonded_out[9].item()) == pytest.approx(np.sum(v.astype(np.float64) ** 2),
                                                          rel=1e-6)
    assert box1 == pytest.approx((box0 * alpha).astype(np.float32).astype(np.float64), rel=1e-7)
    assert np.allclose(r_after, (r_before * alpha).astype(np.float32), rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("targets", [(1.0, 1.0), (1.0, 0.0), (0.0, 1.0)])
def test_semiisotropic_barostat_matches_reference_formula(targets):
    """Semi-isotropic SCR with z normal (hymd/barostat_scr.py:133-284): lateral
    and normal pressures, surface tension, the two scale factors, the box,
    and the reference's row-indexed position update (particles 0 and 1 by
    alpha_L, particle 2 by alpha_N, the rest unchanged); a zero target leaves
    its direction uncoupled."""
    from hymd_gb300 import _lib
    from hymd_gb300.md import RespaMD
    s, cfg, ham = _system()
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    md.couple(thermostat=False, barostat="semiisotropic", seed=6, n_steps=10,
              target_pressure=targets)
    md.prime()
    r_field = md.r.cpu().numpy().copy()
    box0 = md.box_now()
    st = _lib.stream_ptr()
    md._inner_fused(st)
    r_before = md.r.cpu().numpy().copy()
    v = md.v.cpu().numpy()
    bonded = md.bonded_out.cpu().numpy()
    box1 = md.box_now()
    md._outer_rest(st)  # position update, then the field at the new box
    r_after = md.r.cpu().numpy()
    fun = _functional(cfg)
    ref = of.update_field(r_field.astype(np.float64), s["types"], cfg.n_types, cfg.mesh(), box0,
                          cfg.m, fun, cfg.sigma)
    P18 = of.comp_pressure(ref["phi"], ref["phi_fourier"], fun, v, cfg.mass, cfg.mesh(), box0,
                           cfg.sigma, bonded[1:4], bonded[5:8])
    PL = (P18[-3] + P18[-2]) / 2 * 16.61
    PN = P18[-1] * 16.61
    gamma = box0[2] / 2 * (PN - PL)
    Rxy, Rz = md.randoms.cpu().numpy().reshape(10, -1)[0, :2]
    dt_o = cfg.respa_inner * cfg.time_step
    beta, T_, R_ = 7.6e-4, cfg.target_temperature, cfg.gas_constant
    box = box0.astype(np.float32).copy()
    aL = aN = 1.0
    if targets[0]:
        V = np.prod(box.astype(np.float64))
        noise = np.sqrt(4.0 * R_ * T_ * beta * dt_o / (3 * V * cfg.tau_p)) * Rxy
        la = -2.0 * dt_o * beta / (3 * cfg.tau_p) * (targets[0] - PL - gamma / box[2]) + noise
        aL = np.exp(la / 2.0)
        box[0:2] *= aL
    if targets[1]:
        V = np.prod(box.astype(np.float64))
        noise = np.sqrt(2.0 * R_ * T_ * beta * dt_o / (3 * V * cfg.tau_p)) * Rz
        la = -dt_o * beta / (3 * cfg.tau_p) * (targets[1] - PN) + noise
        aN = np.exp(la)
        box[2] *= aN
    state = md.state.cpu().numpy()
    assert state[13] == pytest.approx(PL, rel=1e-5, abs=5e-2)
    assert state[15] == pytest.approx(PN, rel=1e-5, abs=5e-2)
    assert state[10] == pytest.approx(gamma, rel=1e-5, abs=5e-1)
    assert state[12] == pytest.approx(aL, rel=1e-7)
    assert state[14] == pytest.approx(aN, rel=1e-7)
    assert box1 == pytest.approx(box.astype(np.float64), rel=1e-7)
    want = r_before.copy()
    want[0:2] = (r_before[0:2].astype(np.float64) * aL).astype(np.float32)
    want[2] = (r_before[2].astype(np.float64) * aN).astype(np.float32)
    # the field step's paint may wrap nothing here: positions are only rescaled
    assert np.allclose(r_after[:3], want[:3], rtol=1e-6, atol=1e-6)
    assert np.array_equal(r_after[3:], r_before[3:])
    md.check_errors()


def test_coupled_md_graph_runs_and_keeps_temperature():
    from hymd_gb300.md import RespaMD
    s, cfg, ham = _system()
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    md.couple(thermostat=True, barostat="isotropic", seed=1, n_steps=200)
    md.prime()
    md.capture()
    md.run(40)
    torch.cuda.synchronize()
    md.check_errors()
    v = md.v.cpu().numpy().astype(np.float64)
    T = cfg.mass * np.sum(v ** 2) / (3 * len(v) * cfg.gas_constant)
    assert 200.0 < T < 500.0
    assert np.all(np.isfinite(md.r.cpu().numpy()))
    assert int(md.counter[0].item()) == 41
