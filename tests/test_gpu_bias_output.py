"""The PLUMED bias inside the device MD loop, and the asynchronous trajectory
output.

* RespaMD.set_bias with PlumedBias over tests/plumed_fake.py (a DISTANCE
  restraint between two beads of a chain) against the oracle rRESPA loop
  with the same bias applied as hymd/main.py:808-812, 1097-1154 does: two
  outer steps, the same tolerances as the unbiased loop test.
* TrajectoryRecorder (with and without its writer thread): frames every
  n_print steps of a thermostatted membrane run, written through
  file_io.store_data into the in-memory H5 tree, against the state and the
  drop-in energies / pressure taken synchronously at the same steps.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import hamiltonian as oh  # noqa: E402
from oracle import md as omd  # noqa: E402
from plumed_fake import FakePlumed  # noqa: E402


def rel_rms(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def _plumed(cfg, tmp_path, tag):
    from hymd_gb300.plumed import PlumedBias
    dat = os.path.join(tmp_path, f"plumed_{tag}.dat")
    with open(dat, "w") as f:
        # beads 3 and 17 of the first chain pulled to 0.8 nm
        f.write("d: DISTANCE ATOMS=3,17\nRESTRAINT ARG=d KAPPA=4000.0 AT=0.8\n")
    return PlumedBias(cfg, dat, os.path.join(tmp_path, f"log_{tag}"), kernel=FakePlumed())


def test_bias_in_md_loop_matches_oracle(tmp_path):
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    s = systems.homopolymer_melt(seed=11, n_chains=300, length=10, box=6.0, mesh=24)
    cfg = s["config"]
    cfg.target_temperature = 323.0
    ham = get_hamiltonian(cfg)
    fun = oh.quadratic_from_params("DefaultWithChi", 2, cfg.kappa, cfg.rho0, cfg.a,
                                   np.array([[0, 15.0], [15.0, 0]]))
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    md.set_bias(_plumed(cfg, tmp_path, "gpu"))
    md.prime()
    ob = _plumed(cfg, tmp_path, "cpu")
    idx = np.arange(len(s["positions"]), dtype=np.intc)

    def bias(step, r, forces):
        ob.prepare(step, forces, r, idx, cfg, np.zeros(len(r)))
        fb, _ = ob.calc(forces, 0.0)
        return fb

    r = s["positions"].copy()
    v = s["velocities"].copy()
    ff = omd.field_forces(r, s["types"], cfg, fun)
    fbd, fba = omd.bonded_forces(r, s["topology"], cfg.box())
    f_bias = np.asarray(bias(0, r, ff + fbd + fba), np.float32)
    assert rel_rms(md.f_bias.cpu().numpy(), f_bias) < 1e-5
    assert np.count_nonzero(np.abs(f_bias).sum(1)) == 2
    for step in (1, 2):
        md.step()
        r, v, ff, f_bias = omd.respa_step(r, v, ff, s["types"], s["topology"], cfg, fun,
                                          bias=bias, f_bias=f_bias, step=step)
    rg = md.r.cpu().numpy()
    d = np.abs(rg - r)
    d = np.minimum(d, cfg.box()[None, :] - d)
    assert np.sqrt(np.mean(d ** 2)) < 1e-5 * np.sqrt(np.mean(r ** 2))
    assert rel_rms(md.v.cpu().numpy(), v) < 1e-4
    assert rel_rms(md.f_bias.cpu().numpy(), f_bias) < 1e-4
    assert md.plumed_bias > 0.0
    # the bias moved the two beads: the same run without it differs there
    ref = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    ref.prime()
    ref.run(2)
    dv = np.abs(ref.v.cpu().numpy() - md.v.cpu().numpy()).sum(1)
    assert dv[2] > 1e-2 and dv[16] > 1e-2
    with pytest.raises(RuntimeError):
        md.capture()
    md.check_errors()


@pytest.mark.parametrize("threaded", [True, False])
def test_trajectory_recorder_frames(tmp_path, threaded):
    from hymd_gb300 import _lib, systems
    from hymd_gb300 import file_io as fio
    from hymd_gb300.field import energy_fp64
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    from hymd_gb300.pressure import pressure_vector
    from hymd_gb300.trajectory import TrajectoryRecorder
    s = systems.lipid_membrane(seed=4, n_lipids=200, n_water=3000, box=8.0, mesh=24)
    cfg = s["config"]
    cfg.n_steps, cfg.n_print = 12, 4
    ham = get_hamiltonian(cfg)
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    md.sort_particles()
    md.couple(thermostat=True, barostat=None, seed=3, n_steps=50)
    md.prime()
    md.capture()
    n = md.n
    out = fio.OutDataset(str(tmp_path), cfg, backend="memory")
    topo = s["topology"]
    fio.store_static(out, list(range(n)), s["names"], s["types"], np.arange(n), cfg, topo[0],
                     topo[1], molecules=s["molecules"], velocity_out=True, force_out=True)
    rec = TrajectoryRecorder(md, out, ham, velocity_out=True, force_out=True, pressure=True,
                             depth=2, threaded=threaded)
    want = {}

    def expect(step):
        torch.cuda.synchronize()
        r = md.in_input_order(md.r).cpu().numpy()
        v = md.in_input_order(md.v).cpu().numpy()
        f = md.in_input_order(md.f_field + md.f_b).cpu().numpy()
        e = energy_fp64(md.pm, md.r, md.types, cfg.m, ham)
        ke = 0.5 * cfg.mass * float(np.sum(md.v.double().cpu().numpy() ** 2))
        bo = md.bonded_out.cpu().numpy()
        P = pressure_vector(e, ke, bo[1:4], bo[5:8])
        want[step] = dict(r=r, v=v, f=f, W=e["W"], ke=ke, P=P, box=md.box_now(),
                          work=float(md.state[8].item() + md.state[9].item()), eb=bo[[0, 4, 8]])

    rec.record(0)
    expect(0)
    for step in range(1, cfg.n_steps + 1):
        md.run(1)
        if step % cfg.n_print == 0:
            rec.record(step)
            expect(step)
        rec.drain()
    rec.close()
    assert rec.written == 4
    if threaded:
        with pytest.raises(RuntimeError):
            rec.record(cfg.n_steps + cfg.n_print)
    for frame, step in enumerate(sorted(want)):
        w = want[step]
        assert out.positions_step[frame] == step
        assert out.positions_time[frame] == pytest.approx(step * cfg.respa_inner * cfg.time_step,
                                                          rel=1e-6)
        assert np.array_equal(out.positions[frame], w["r"])
        assert np.array_equal(out.velocities[frame], w["v"])
        assert rel_rms(out.forces[frame], w["f"]) < 1e-6
        assert out.field_energy[frame][0] == pytest.approx(w["W"], rel=1e-6)
        assert out.kinetc_energy[frame][0] == pytest.approx(w["ke"], rel=1e-6)
        assert out.bond_energy[frame][0] == pytest.approx(w["eb"][0], rel=1e-6)
        assert out.angle_energy[frame][0] == pytest.approx(w["eb"][1], rel=1e-6)
        T = (2.0 / 3.0) * w["ke"] / (cfg.gas_constant * n)
        assert out.temperature[frame][0] == pytest.approx(T, rel=1e-6)
        assert np.allclose(out.pressure[frame], w["P"], rtol=1e-5, atol=1e-5 * np.abs(w["P"]).max())
        assert np.allclose(np.diag(out.box_value[frame]), w["box"], rtol=1e-6)
        assert out.thermostat_work[frame][0] == pytest.approx(w["work"], rel=1e-5, abs=1e-3)
    md.check_errors()
