"""The FP64 oracle against outputs of the reference's own code.

tests/golden/field_ref.npz was written by tests/golden/make_field_ref.py,
which ran the unmodified hymd/field.py, pressure.py, thermostat.py and
barostat_scr.py (through a numpy stand-in for the pmesh library the reference
takes as an argument).  Both sides are FP64, so the tolerances here are
round-off level: forces, grids, energies and pressure within 1e-9 relative
(the stand-in's and the oracle's Nyquist conventions differ only below
exp(-sigma^2 k_N^2) ~ 1e-11 on these meshes); coupling results within 1e-12.
"""
import os

import numpy as np
import pytest

from oracle import coupling as oc
from oracle import field as of
from oracle import hamiltonian as oh

FIX = np.load(os.path.join(os.path.dirname(__file__), "golden", "field_ref.npz"))
FP64_RTOL = 1e-9


def rel_rms(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def case(pre):
    d = {k[len(pre):]: FIX[k] for k in FIX.files if k.startswith(pre)}
    sigma, kappa, mass, rho0, a = d["scalars"]
    d.update(sigma=sigma, kappa=kappa, mass=mass, rho0=rho0, a=a)
    return d


def functional(d, kind="DefaultWithChi"):
    T = len(d["m"])
    return oh.quadratic_from_params(kind, T, d["kappa"], d["rho0"], d["a"], d["chi"])


def oracle_field(d, kind):
    T = len(d["m"])
    fun = functional(d, kind)
    r = d["positions"].astype(np.float64)
    out = of.update_field(r, d["types"], T, d["mesh"], d["box"], d["m"], fun, d["sigma"],
                          compute_potential=True)
    F = of.compute_field_force(out["force_mesh"], r, d["types"], T, d["mesh"], d["box"])
    return fun, out, F


@pytest.mark.parametrize("name", ["chi3_cubic", "chi3_ragged", "nochi2", "sqphi2"])
def test_field_forces_energies_pressure_match_reference(name):
    d = case(f"field/{name}/")
    kind = str(d["kind"])
    fun, out, F = oracle_field(d, kind)
    assert rel_rms(F, d["forces"]) < FP64_RTOL
    W = of.field_energy(out["phi"], fun, d["mesh"], d["box"])
    KE = of.kinetic_energy(d["velocities"], d["mass"])
    assert W == pytest.approx(d["energies"][0], rel=FP64_RTOL)
    assert KE == pytest.approx(d["energies"][1], rel=1e-12)
    P = of.comp_pressure(out["phi"], out["phi_fourier"], fun, d["velocities"], d["mass"],
                         d["mesh"], d["box"], d["sigma"], d["bond_pr"], d["angle_pr"])
    assert np.allclose(P, d["pressure"], rtol=FP64_RTOL, atol=FP64_RTOL * np.abs(d["pressure"]).max())
    if "phi" in d:
        assert rel_rms(np.stack(out["phi"]), d["phi"]) < FP64_RTOL
        assert rel_rms(np.stack(out["v_ext"]), d["v_ext"]) < FP64_RTOL


def test_pic_matches_reference():
    d = case("pic/")
    fun, out, F = oracle_field(d, "DefaultWithChi")
    r = d["positions"].astype(np.float64)
    eps = float(d["dielectric_const"])
    q = of.update_field_force_q(d["charges"], r, d["mesh"], d["box"], d["sigma"], eps)
    assert rel_rms(F, d["forces"]) < FP64_RTOL
    assert rel_rms(q["forces"], d["elec_forces"]) < FP64_RTOL
    assert rel_rms(q["psi"], d["psi"]) < FP64_RTOL
    Es = of.self_energy_q(d["charges"], d["sigma"], eps)
    assert Es == pytest.approx(float(d["self_energy"]), rel=1e-12)
    Wq = of.field_q_energy(q["phi_q"], q["psi"], Es, d["mesh"], d["box"])
    assert Wq == pytest.approx(d["energies"][2], rel=FP64_RTOL)
    P = of.comp_pressure(out["phi"], out["phi_fourier"], fun, d["velocities"], d["mass"],
                         d["mesh"], d["box"], d["sigma"], d["bond_pr"], d["angle_pr"],
                         phi_q=q["phi_q"], psi=q["psi"], self_energy=Es,
                         type_charges=d["type_charges"])
    assert np.allclose(P, d["pressure"], rtol=FP64_RTOL, atol=FP64_RTOL * np.abs(d["pressure"]).max())


def test_gpe_two_calls_match_reference():
    """Both calls start the polarisation iteration from zero (the reference's
    caller grid never changes), so both take the same number of iterations.
    The iteration forms eta . E and q / eps in real space with no filter, so
    Nyquist content survives and the stand-in's Nyquist convention shows at
    ~2e-8: the tolerance here is 1e-7."""
    d = case("gpe/")
    T = len(d["m"])
    fun = functional(d)
    nshape = tuple(int(x) for x in d["mesh"])
    state = dict(phi_eps=np.zeros(nshape), pol_prev=np.zeros(nshape), contrib=np.zeros(nshape))
    for call, key in enumerate(("positions", "positions2")):
        r = d[key].astype(np.float64)
        fld = of.update_field(r, d["types"], T, d["mesh"], d["box"], d["m"], fun, d["sigma"])
        g = of.gpe_step(fld["phi"], d["charges"], r, d["types"], T, d["mesh"], d["box"],
                        d["sigma"], d["dielectric_type"], d["type_charges"], state,
                        conv_crit=d["conv"][0], mixing=d["conv"][1], conv_kind="max_diff")
        c = f"call{call}/"
        assert g["iterations"] == int(d[c + "iterations"])
        assert rel_rms(g["forces"], d[c + "elec_forces"]) < 1e-7
        assert rel_rms(g["psi"], d[c + "psi"]) < 1e-7
        assert rel_rms(g["phi_eps"], d[c + "phi_eps"]) < 1e-12
        assert g["energy"] == pytest.approx(float(d[c + "energy"]), rel=1e-7)


@pytest.mark.parametrize("name", ["one_com", "one_nocom", "two_com", "two_nocom"])
def test_csvr_matches_reference(name):
    d = {k.split("/")[-1]: FIX[k] for k in FIX.files if k.startswith(f"csvr/{name}/")}
    mass, gas, temp, dt_o, tau = d["params"]
    ng = int(d["group"].max()) + 1
    v, work = oc.csvr(d["v0"], d["group"], ng, mass, temp, dt_o, tau, d["draws"],
                      remove_com=name.endswith("_com"), gas_constant=gas)
    assert np.allclose(v, d["v1"], rtol=1e-12, atol=1e-14)
    assert work == pytest.approx(float(d["work"]), rel=1e-12)


@pytest.mark.parametrize("mode", ["iso", "semi", "semi_lateral"])
def test_scr_matches_reference(mode):
    d = case(f"scr/{mode}/")
    fun, out, F = oracle_field(d, "DefaultWithChi")
    P = of.comp_pressure(out["phi"], out["phi_fourier"], fun, d["velocities"], d["mass"],
                         d["mesh"], d["box"], d["sigma"], d["bond_pr"], d["angle_pr"])
    assert np.allclose(P, d["pressure"], rtol=FP64_RTOL, atol=FP64_RTOL * np.abs(d["pressure"]).max())
    tau_p, n_b, dt_o, temp, gas = d["params"]
    r = d["positions"].astype(np.float64)
    if mode == "iso":
        box, pos, _ = oc.scr_isotropic(d["pressure"], d["box"], r, d["draws"][0], d["targets"][0],
                                       tau_p, n_b, dt_o, temp, gas)
    else:
        box, pos, _, _, _ = oc.scr_semiisotropic(d["pressure"], d["box"], r, d["draws"][0],
                                                 d["draws"][1], d["targets"][0], d["targets"][1],
                                                 tau_p, n_b, dt_o, temp, gas)
    assert np.allclose(box, d["box_after"], rtol=1e-14)
    assert np.allclose(pos, d["positions_after"], rtol=1e-14)
