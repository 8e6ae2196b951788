"""Generate tests/golden/field_ref.npz by running the reference's own field,
pressure, thermostat and barostat code.

    python tests/golden/make_field_ref.py <path-to-HyMD-checkout>
    (or set HYMD_REFERENCE)

The unmodified modules hymd/field.py, hymd/pressure.py, hymd/hamiltonian.py,
hymd/thermostat.py, hymd/barostat_scr.py and hymd/input_parser.py (Config)
are loaded by file path, with the stubs of make_golden.py (one-rank mpi4py,
empty h5py / f2py modules) and with `pmesh_standin` passed as the `pmesh`
module to the reference's own `initialize_pm` (hymd/field.py:10-149) -- the
reference takes the mesh library as an argument, so nothing in it is patched.
Everything runs in float64 (config.dtype = np.float64, pmesh dtype "f8").

Cases (keys are prefixed by the case name):
  field/<name>  update_field (hymd/field.py:428-616, compute_potential=True),
                compute_field_force (:152-200), compute_field_and_kinetic_energy
                (:619-703) and comp_pressure (hymd/pressure.py:9-179) for the
                DefaultWithChi (cubic 16^3 and ragged 12x16x20 meshes),
                DefaultNoChi and SquaredPhi functionals
  pic           update_field_force_q (PIC_Spectral, :241-403), the electrostatic
                energy, compute_self_energy_q (:203-238) and the pressure with
                the electrostatic V_bar
  gpe           update_field_force_q_GPE (:764-1112) and
                compute_field_energy_q_GPE (:706-761) called twice in a row on
                the same grids (second call at displaced positions), with the
                iteration counts of each call
  csvr/<name>   csvr_thermostat (hymd/thermostat.py:111-219) for one and two
                coupling groups, with and without centre-of-mass removal; the
                random draws are recorded
  scr/<name>    isotropic and semiisotropic SCR steps (hymd/barostat_scr.py:
                34-284): pressure, box and positions after, the draws

The meshes keep h <= 0.3125 nm with sigma = 0.5 nm, so the doubly filtered
Nyquist modes of the field forces are below exp(-sigma^2 k_N^2) ~ 1e-11 of
the signal; the electrostatic cases, filtered once and divided by k^2, use
h = 0.25 nm (exp(-sigma^2 k_N^2 / 2) (k_1 / k_N)^2 ~ 1e-11).  So the
stand-in's Nyquist convention does not show (pmesh_standin.py).
"""
import os
import sys
import types as _types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import make_golden as mg  # noqa: E402
import pmesh_standin  # noqa: E402


def _load_reference(ref):
    import warnings
    warnings.filterwarnings("ignore", category=SyntaxWarning)
    mg._install_stubs()
    pkg = _types.ModuleType("hymd")
    pkg.__path__ = [os.path.join(ref, "hymd")]
    sys.modules["hymd"] = pkg
    mods = {}
    for name in ("version", "logger", "force", "barostat", "input_parser", "hamiltonian",
                 "field", "pressure", "thermostat", "barostat_scr"):
        mods[name] = mg._load("hymd." + name, os.path.join(ref, "hymd", name + ".py"), "hymd")
    return mods


def _system(rng, n, T, box, counts=None, cluster=0.35):
    box = np.asarray(box, np.float64)
    r = rng.uniform(0, 1, (n, 3)) * box
    k = int(cluster * n)
    r[:k] = np.mod(box / 2 + rng.normal(0, 0.6, (k, 3)), box)
    r = r.astype(np.float32)
    if counts is None:
        types = rng.integers(0, T, n).astype(np.int64)
    else:
        types = np.concatenate([np.full(c, t) for t, c in enumerate(counts)]).astype(np.int64)
        types = types[rng.permutation(n)]
    v = rng.normal(0, 0.3, (n, 3)).astype(np.float32)
    return r, types, v


def _config(R, mesh, box, n, T, kind, rng, chi_names=None, **extra):
    Config = R["input_parser"].Config
    Chi = R["force"].Chi
    names = [chr(65 + t) for t in range(T)]
    cfg = Config(n_steps=1, time_step=0.03, mesh_size=np.asarray(mesh), sigma=0.5, kappa=0.05,
                 dtype=np.float64, box_size=np.asarray(box, np.float64), n_particles=n,
                 mass=72.0, hamiltonian=kind, respa_inner=10, tau=0.1,
                 target_temperature=323.0)
    cfg.n_types = T
    cfg.unique_names = names
    cfg.type_to_name_map = dict(enumerate(names))
    cfg.chi = [Chi(atom_1=names[i], atom_2=names[j],
                   interaction_energy=float(rng.uniform(2.0, 25.0)))
               for i in range(T) for j in range(i + 1, T)]
    cfg.m = [float(x) for x in rng.uniform(0.8, 1.2, T)]
    cfg.type_charges = [0.0] * T
    for key, val in extra.items():
        setattr(cfg, key, val)
    return cfg, names


def _chi_matrix(cfg, names):
    T = len(names)
    chi = np.zeros((T, T))
    for c in cfg.chi:
        i, j = names.index(c.atom_1), names.index(c.atom_2)
        chi[i, j] = chi[j, i] = c.interaction_energy
    return chi


def _common(out, pre, cfg, names, r, types, v):
    out[pre + "positions"] = r
    out[pre + "types"] = types
    out[pre + "velocities"] = v
    out[pre + "box"] = np.asarray(cfg.box_size, np.float64).copy()
    out[pre + "mesh"] = np.asarray(cfg.mesh_size, np.int64)
    out[pre + "m"] = np.asarray(cfg.m, np.float64)
    out[pre + "chi"] = _chi_matrix(cfg, names)
    out[pre + "scalars"] = np.array([cfg.sigma, cfg.kappa, cfg.mass, cfg.rho0, cfg.a])


def field_case(R, out, name, kind, T, box, mesh, seed, n=2400, store_grids=False):
    rng = np.random.default_rng(seed)
    r, types, v = _system(rng, n, T, box)
    cfg, names = _config(R, mesh, box, n, T, kind, rng)
    ham = R["hamiltonian"].get_hamiltonian(cfg)
    F = R["field"]
    pm, fl, ecl, cl = F.initialize_pm(pmesh_standin, cfg)
    phi, phi_fourier, force_on_grid, v_ext_fourier, v_ext, phi_transfer, phi_lap = fl
    pos = r.astype(np.float64)
    layouts = [None] * T
    F.update_field(phi, phi_lap, phi_transfer, layouts, force_on_grid, ham, pm, pos, types, cfg,
                   v_ext, phi_fourier, v_ext_fourier, cfg.m, compute_potential=True)
    force = np.zeros((n, 3))
    F.compute_field_force(layouts, pos, force_on_grid, force, types, T)
    vel = v.astype(np.float64)
    W, KE, Wq = F.compute_field_and_kinetic_energy(phi, None, None, vel, ham, pos, types, v_ext,
                                                   cfg, layouts)
    bond_pr = rng.normal(0, 50.0, 3)
    angle_pr = rng.normal(0, 20.0, 3)
    P = R["pressure"].comp_pressure(phi, None, None, ham, vel, cfg, phi_fourier, phi_lap,
                                    phi_transfer, pos, bond_pr, angle_pr)
    pre = f"field/{name}/"
    _common(out, pre, cfg, names, r, types, v)
    out[pre + "kind"] = np.array(kind)
    out[pre + "forces"] = force
    out[pre + "energies"] = np.array([W, KE, Wq])
    out[pre + "bond_pr"] = bond_pr
    out[pre + "angle_pr"] = angle_pr
    out[pre + "pressure"] = np.asarray(P, np.float64)
    if store_grids:
        out[pre + "phi"] = np.stack([p.value for p in phi])
        out[pre + "v_ext"] = np.stack([p.value for p in v_ext])
    print(name, kind, "W", W, "KE", KE, "|F| rms", np.sqrt(np.mean(force ** 2)))


def pic_case(R, out, seed=21, n=2400):
    rng = np.random.default_rng(seed)
    T, box, mesh = 3, (4.0, 4.0, 4.0), (16, 16, 16)
    counts = [n - 400, 200, 200]
    r, types, v = _system(rng, n, T, box, counts=counts)
    type_charges = [0.0, 1.0, -1.0]
    charges = np.asarray(type_charges)[types]
    cfg, names = _config(R, mesh, box, n, T, "DefaultWithChi", rng, coulombtype="PIC_Spectral",
                         dielectric_const=80.0, type_charges=type_charges)
    F = R["field"]
    cfg.self_energy = F.compute_self_energy_q(cfg, charges)
    ham = R["hamiltonian"].get_hamiltonian(cfg)
    pm, fl, ecl, cl = F.initialize_pm(pmesh_standin, cfg)
    phi, phi_fourier, force_on_grid, v_ext_fourier, v_ext, phi_transfer, phi_lap = fl
    phi_q, phi_q_fourier, psi, elec_field = ecl
    elec_field_fourier, psi_fourier = cl
    pos = r.astype(np.float64)
    layouts = [None] * T
    F.update_field(phi, phi_lap, phi_transfer, layouts, force_on_grid, ham, pm, pos, types, cfg,
                   v_ext, phi_fourier, v_ext_fourier, cfg.m, compute_potential=True)
    force = np.zeros((n, 3))
    F.compute_field_force(layouts, pos, force_on_grid, force, types, T)
    elec_forces = np.zeros((n, 3))
    F.update_field_force_q(charges, phi_q, phi_q_fourier, psi, psi_fourier, elec_field_fourier,
                           elec_field, elec_forces, None, ham, pm, pos, cfg)
    vel = v.astype(np.float64)
    W, KE, Wq = F.compute_field_and_kinetic_energy(phi, phi_q, psi, vel, ham, pos, types, v_ext,
                                                   cfg, layouts)
    bond_pr = rng.normal(0, 50.0, 3)
    angle_pr = rng.normal(0, 20.0, 3)
    P = R["pressure"].comp_pressure(phi, phi_q, psi, ham, vel, cfg, phi_fourier, phi_lap,
                                    phi_transfer, pos, bond_pr, angle_pr)
    pre = "pic/"
    _common(out, pre, cfg, names, r, types, v)
    out[pre + "charges"] = charges
    out[pre + "type_charges"] = np.asarray(type_charges)
    out[pre + "dielectric_const"] = np.array(cfg.dielectric_const)
    out[pre + "self_energy"] = np.array(cfg.self_energy)
    out[pre + "forces"] = force
    out[pre + "elec_forces"] = elec_forces
    out[pre + "psi"] = psi.value.copy()
    out[pre + "energies"] = np.array([W, KE, Wq])
    out[pre + "bond_pr"] = bond_pr
    out[pre + "angle_pr"] = angle_pr
    out[pre + "pressure"] = np.asarray(P, np.float64)
    print("pic W", W, "Wq", Wq, "E_self", cfg.self_energy,
          "|F_el| rms", np.sqrt(np.mean(elec_forces ** 2)))


def gpe_case(R, out, seed=33, n=2400):
    rng = np.random.default_rng(seed)
    T, box, mesh = 3, (4.0, 4.0, 4.0), (16, 16, 16)
    counts = [n - 400, 200, 200]
    r, types, v = _system(rng, n, T, box, counts=counts, cluster=0.2)
    type_charges = [0.0, 1.0, -1.0]
    charges = np.asarray(type_charges)[types]
    eps_type = [80.0, 20.0, 40.0]
    cfg, names = _config(R, mesh, box, n, T, "DefaultWithChi", rng,
                         coulombtype="PIC_Spectral_GPE", type_charges=type_charges,
                         dielectric_type=eps_type, conv_crit=1e-6, pol_mixing=0.6,
                         convergence_type="max_diff")
    F = R["field"]
    ham = R["hamiltonian"].get_hamiltonian(cfg)
    pm, fl, ecl, cl = F.initialize_pm(pmesh_standin, cfg)
    phi, phi_fourier, force_on_grid, v_ext_fourier, v_ext, phi_transfer, phi_lap = fl
    phi_q, phi_q_fourier, psi, elec_field = ecl
    (phi_eps, phi_eps_fourier, phi_eta, phi_eta_fourier, phi_pol, phi_pol_prev, elec_dot,
     elec_field_contrib, Vbar_elec, Vbar_elec_fourier, force_mesh_elec,
     force_mesh_elec_fourier) = cl
    calls = []

    def conv_fun(comm, diffmesh):
        # the default convergence measure of hymd/main.py:154-165 (max_diff)
        calls.append(1)
        return np.max(diffmesh)

    pre = "gpe/"
    _common(out, pre, cfg, names, r, types, v)
    out[pre + "charges"] = charges
    out[pre + "type_charges"] = np.asarray(type_charges)
    out[pre + "dielectric_type"] = np.asarray(eps_type)
    out[pre + "conv"] = np.array([cfg.conv_crit, cfg.pol_mixing])
    pos = r.astype(np.float64)
    layouts = [None] * T
    for call in range(2):
        if call == 1:
            pos = np.mod(pos + rng.normal(0, 0.05, pos.shape), np.asarray(box)).astype(
                np.float32).astype(np.float64)
            out[pre + "positions2"] = pos.astype(np.float32)
        F.update_field(phi, phi_lap, phi_transfer, layouts, force_on_grid, ham, pm, pos, types,
                       cfg, v_ext, phi_fourier, v_ext_fourier, cfg.m, compute_potential=True)
        elec_forces = np.zeros((n, 3))
        calls.clear()
        Vb, pe, dot = F.update_field_force_q_GPE(
            conv_fun, phi, types, charges, phi_q, phi_q_fourier, phi_eps, phi_eps_fourier,
            phi_eta, phi_eta_fourier, phi_pol_prev, phi_pol, elec_field, elec_forces,
            elec_field_contrib, psi, Vbar_elec, Vbar_elec_fourier, force_mesh_elec,
            force_mesh_elec_fourier, ham, None, layouts, pm, pos, cfg)
        Eq = F.compute_field_energy_q_GPE(cfg, pe, 0.0, dot)
        c = f"{pre}call{call}/"
        out[c + "elec_forces"] = elec_forces
        out[c + "psi"] = psi.value.copy()
        out[c + "phi_eps"] = pe.value.copy()
        out[c + "energy"] = np.array(Eq)
        out[c + "iterations"] = np.array(len(calls))
        print("gpe call", call, "iterations", len(calls), "energy", Eq,
              "|F_el| rms", np.sqrt(np.mean(elec_forces ** 2)))


def csvr_cases(R, out, seed=41, n=600):
    Th = R["thermostat"]
    rng = np.random.default_rng(seed)
    names_all = np.array([b"A", b"B", b"C"])[rng.integers(0, 3, n)]
    v0 = rng.normal(0, 0.4, (n, 3)) + np.array([0.05, -0.02, 0.03])
    groups_list = {"one": [["A", "B", "C"]], "two": [["A", "B"], ["C"]]}
    for gname, groups in groups_list.items():
        for com in (True, False):
            Config = R["input_parser"].Config
            cfg = Config(n_steps=1, time_step=0.03, mesh_size=[8, 8, 8], sigma=0.5, kappa=0.05,
                         box_size=np.array([5.0, 5.0, 5.0]), mass=72.0, respa_inner=10,
                         tau=0.1, target_temperature=323.0)
            cfg.unique_names = ["A", "B", "C"]
            cfg.thermostat_coupling_groups = [list(g) for g in groups]
            cfg.thermostat_work = 0.0
            draws = []

            def gauss(prng):
                x = prng.normal()
                draws.append(x)
                return x

            def chi2(prng, M):
                x = prng.chisquare(M)
                draws.append(x)
                return x

            v = v0.copy()
            Th.csvr_thermostat(v, names_all, cfg, np.random.default_rng(seed + 7), random_gaussian=gauss,
                               random_chi_squared=chi2, remove_center_of_mass_momentum=com)
            pre = f"csvr/{gname}_{'com' if com else 'nocom'}/"
            gid = np.zeros(n, np.int32)
            for gi, g in enumerate(groups):
                for nm in g:
                    gid[names_all == nm.encode()] = gi
            out[pre + "v0"] = v0
            out[pre + "v1"] = v
            out[pre + "group"] = gid
            out[pre + "draws"] = np.asarray(draws)
            out[pre + "work"] = np.array(cfg.thermostat_work)
            out[pre + "params"] = np.array([cfg.mass, cfg.gas_constant, cfg.target_temperature,
                                            cfg.time_step * cfg.respa_inner, cfg.tau])
            print("csvr", gname, com, "work", cfg.thermostat_work)


def scr_cases(R, out, seed=51, n=2400):
    B = R["barostat_scr"]
    Tp = R["barostat"].Target_pressure
    for mode, targets in (("iso", (1.0, None)), ("semi", (1.0, 1.0)), ("semi_lateral", (1.0, 0))):
        rng = np.random.default_rng(seed)
        T, box = 3, (5.0, 5.0, 5.0)
        mesh = (16, 16, 16)
        r, types, v = _system(rng, n, T, box)
        V = float(np.prod(box))
        cfg, names = _config(R, mesh, box, n, T, "DefaultWithChi", rng,
                             barostat="isotropic" if mode == "iso" else "semiisotropic",
                             barostat_type="scr", tau_p=20.0, n_b=1,
                             target_pressure=Tp(P_L=targets[0], P_N=targets[1]),
                             rho0=n / V, a=n / V)
        ham = R["hamiltonian"].get_hamiltonian(cfg)
        F = R["field"]
        pm_stuff = F.initialize_pm(pmesh_standin, cfg)
        pm, fl, ecl, cl = pm_stuff
        phi, phi_fourier, force_on_grid, v_ext_fourier, v_ext, phi_transfer, phi_lap = fl
        pos = r.astype(np.float64)
        layouts = [None] * T
        F.update_field(phi, phi_lap, phi_transfer, layouts, force_on_grid, ham, pm, pos, types,
                       cfg, v_ext, phi_fourier, v_ext_fourier, cfg.m, compute_potential=True)
        vel = v.astype(np.float64)
        bond_pr = rng.normal(0, 500.0, 3)
        angle_pr = rng.normal(0, 200.0, 3)
        P = R["pressure"].comp_pressure(phi, None, None, ham, vel, cfg, phi_fourier, phi_lap,
                                        phi_transfer, pos, bond_pr, angle_pr)
        pre = f"scr/{mode}/"
        _common(out, pre, cfg, names, r, types, v)
        out[pre + "bond_pr"] = bond_pr
        out[pre + "angle_pr"] = angle_pr
        out[pre + "pressure"] = np.asarray(P, np.float64)
        out[pre + "targets"] = np.array([targets[0] or 0.0, targets[1] or 0.0])
        out[pre + "params"] = np.array([cfg.tau_p, cfg.n_b, cfg.time_step * cfg.respa_inner,
                                        cfg.target_temperature, cfg.gas_constant])
        prng = np.random.default_rng(seed + 100)
        out[pre + "draws"] = np.random.default_rng(seed + 100).normal(size=2)
        fn = B.isotropic if mode == "iso" else B.semiisotropic
        pos_after = pos.copy()
        fn(pmesh_standin, pm_stuff, phi, None, None, ham, pos_after, vel, cfg, phi_fourier,
           phi_lap, phi_transfer, bond_pr, angle_pr, 0, prng)
        out[pre + "box_after"] = np.asarray(cfg.box_size, np.float64).copy()
        out[pre + "positions_after"] = pos_after
        print("scr", mode, "P", P[-3:], "box", cfg.box_size)


def main(ref):
    R = _load_reference(ref)
    out = {}
    field_case(R, out, "chi3_cubic", "DefaultWithChi", 3, (5.0, 5.0, 5.0), (16, 16, 16), 1,
               store_grids=True)
    field_case(R, out, "chi3_ragged", "DefaultWithChi", 3, (3.75, 5.0, 6.25), (12, 16, 20), 2)
    field_case(R, out, "nochi2", "DefaultNoChi", 2, (5.0, 5.0, 5.0), (16, 16, 16), 3)
    field_case(R, out, "sqphi2", "SquaredPhi", 2, (5.0, 5.0, 5.0), (16, 16, 16), 4)
    pic_case(R, out)
    gpe_case(R, out)
    csvr_cases(R, out)
    scr_cases(R, out)
    path = os.path.join(HERE, "field_ref.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes,", len(out), "arrays")


if __name__ == "__main__":
    main(mg.reference_root())
