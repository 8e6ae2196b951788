"""Generate the golden fixtures in tests/golden/ from the HyMD reference.

Run in a container that has the reference checkout (read-only is fine),
passing its root directory (or setting HYMD_REFERENCE):

    python tests/golden/make_golden.py <path-to-HyMD-checkout>

It imports the reference's own pure-Python modules by file path (bypassing
hymd/__init__.py, which pulls in MPI/HDF5/pmesh), with these stubs:
  * mpi4py -> a one-rank communicator (allreduce/bcast are identities)
  * h5py, force_kernels (the f2py extension) -> empty modules
  * pytest.fixture -> identity, so test/conftest.py fixtures are plain functions
and reads the expected vectors of test/test_force.py and test/test_integrator.py
with `ast` (they are local variables of the test functions).

Outputs (all small .npz files):
  topology.npz     prepare_bonds_old / prepare_bonds results (dppc_single,
                   alanine_octapeptide, molecules_with_solvent)
  bonded_kat.npz   the test_force.py expected energies/forces (1e-13 KATs)
  hamiltonian.npz  w_0 / v_ext / V_bar_0 of SquaredPhi, DefaultNoChi and
                   DefaultWithChi evaluated by the reference lambdas on seeded grids
  misc.npz         dipole_forces_redistribution, propensity_potential_coeffs
                   and integrator outputs of the reference (the CSVR thermostat
                   is pinned by make_field_ref.py)
  topology_random.npz  prepare_bonds_old / prepare_bonds on seeded random
                   molecules (branches, rings, scrambled ids, duplicate and
                   reversed term types; random_molecules())
"""
import ast
import importlib.util
import os
import sys
import types as _types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class _Comm:
    def allreduce(self, sendobj=None, op=None):
        return sendobj

    def bcast(self, x, root=0):
        return x

    def gather(self, x, root=0):
        return [x]

    def allgather(self, x):
        return [x]

    def Get_rank(self):
        return 0

    def Get_size(self):
        return 1

    def Barrier(self):
        pass


def _install_stubs():
    mpi = _types.ModuleType("mpi4py")
    MPI = _types.ModuleType("mpi4py.MPI")
    MPI.COMM_WORLD = _Comm()
    MPI.SUM = None
    MPI.Intracomm = _Comm
    mpi.MPI = MPI
    sys.modules["mpi4py"] = mpi
    sys.modules["mpi4py.MPI"] = MPI
    sys.modules["h5py"] = _types.ModuleType("h5py")
    fk = _types.ModuleType("force_kernels")
    for name in ("cbf", "caf", "cdf", "cbf_d", "caf_d", "cdf_d"):
        setattr(fk, name, None)
    sys.modules["force_kernels"] = fk
    tomli = _types.ModuleType("tomli")
    import tomllib
    tomli.loads = tomllib.loads
    sys.modules.setdefault("tomli", tomli)
    import pytest
    pytest.fixture = lambda *a, **k: (a[0] if a and callable(a[0]) else (lambda f: f))
    if not hasattr(np, "string_"):
        np.string_ = np.bytes_
    if not hasattr(np, "VisibleDeprecationWarning"):  # moved to np.exceptions in numpy 2
        np.VisibleDeprecationWarning = np.exceptions.VisibleDeprecationWarning


def _load(name, path, package=None):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    if package:
        mod.__package__ = package
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def _ast_arrays(path, func, names):
    """Evaluate the `name = np.array(...)` assignments inside test function `func`."""
    tree = ast.parse(open(path).read())
    out = {}
    for node in ast.walk(tree):
        if isinstance(node, ast.FunctionDef) and node.name == func:
            for st in node.body:
                if isinstance(st, ast.Assign) and isinstance(st.targets[0], ast.Name):
                    nm = st.targets[0].id
                    if nm in names:
                        out[nm] = eval(compile(ast.Expression(st.value), path, "eval"),
                                       {"np": np})
    return out


def main(ref):
    _install_stubs()
    pkg = _types.ModuleType("hymd")
    pkg.__path__ = [os.path.join(ref, "hymd")]
    sys.modules["hymd"] = pkg
    logger = _load("hymd.logger", os.path.join(ref, "hymd", "logger.py"), "hymd")
    force = _load("hymd.force", os.path.join(ref, "hymd", "force.py"), "hymd")
    force.Logger = logger.Logger
    import logging
    force.logging = logging
    ham = _load("hymd.hamiltonian", os.path.join(ref, "hymd", "hamiltonian.py"), "hymd")
    integ = _load("hymd.integrator", os.path.join(ref, "hymd", "integrator.py"), "hymd")
    conft = _load("ref_conftest", os.path.join(ref, "test", "conftest.py"))

    # ---------------- topology (prepare_bonds_old / prepare_bonds) -------------
    topo = {}

    class Cfg:
        pass

    for fixture in ("dppc_single", "alanine_octapeptide"):
        indices, bonds, names, molecules, r, CONF = getattr(conft, fixture)()
        cfg = Cfg()
        cfg.bonds = list(CONF["bond_2"])
        cfg.angle_bonds = list(CONF["bond_3"])
        cfg.dihedrals = list(CONF.get("bond_4", ()))
        b2, b3, b4, bbi = force.prepare_bonds_old(molecules, names, bonds, indices, cfg)
        packed = force.prepare_bonds(molecules, names, bonds, indices, cfg)
        topo[f"{fixture}/r"] = r
        topo[f"{fixture}/bonds"] = bonds
        topo[f"{fixture}/names"] = names
        topo[f"{fixture}/molecules"] = molecules
        topo[f"{fixture}/indices"] = indices
        topo[f"{fixture}/L"] = np.asarray(CONF["L"], dtype=np.float64)
        topo[f"{fixture}/b2_list"] = np.array([[x[0], x[1], x[2], x[3]] for x in b2], dtype=np.float64)
        topo[f"{fixture}/b3_list"] = np.array([[x[0], x[1], x[2], x[3], x[4]] for x in b3], dtype=np.float64)
        topo[f"{fixture}/b4_idx"] = np.array([[x[0], x[1], x[2], x[3], x[5]] for x in b4], dtype=np.int64).reshape(-1, 5)
        topo[f"{fixture}/bb_index"] = np.asarray(bbi, dtype=np.int64)
        keys = ["b2a", "b2b", "b2r0", "b2k", "b3a", "b3b", "b3c", "b3t0", "b3k",
                "b4a", "b4b", "b4c", "b4d", "b4coeff", "b4type", "b4last"]
        for k, v in zip(keys, packed):
            topo[f"{fixture}/packed/{k}"] = np.asarray(v)

    # molecules_with_solvent: a 4-type system with bonded molecules and free solvent
    idx, r, molecules, vel, bonds, names, types = conft.molecules_with_solvent()
    cfg = Cfg()
    B = force.Bond
    A = force.Angle
    uniq = sorted(set(n.decode() for n in names))
    cfg.bonds = [B(x, y, 0.5, 1000.0) for i, x in enumerate(uniq) for y in uniq[i:]]
    cfg.angle_bonds = [A(atom_1=x, atom_2=y, atom_3=z, equilibrium=120.0, strength=25.0)
                       for x in uniq for y in uniq for z in uniq if x <= z]
    cfg.dihedrals = []
    packed = force.prepare_bonds(molecules, names, bonds, idx, cfg)
    topo["mws/r"] = r
    topo["mws/bonds"] = bonds
    topo["mws/names"] = names
    topo["mws/molecules"] = molecules
    topo["mws/indices"] = idx
    topo["mws/types"] = types
    for k, v in zip(["b2a", "b2b", "b2r0", "b2k", "b3a", "b3b", "b3c", "b3t0", "b3k"], packed[:9]):
        topo[f"mws/packed/{k}"] = np.asarray(v)
    np.savez(os.path.join(HERE, "topology.npz"), **topo)

    # ---------------- bonded known answers (test/test_force.py) ----------------
    tf = os.path.join(ref, "test", "test_force.py")
    kat = {}
    for func, names_ in (
        ("test_comp_bonds", ["expected_energies", "expected_forces_i", "expected_forces_j"]),
        ("test_comp_angles", ["expected_energies", "expected_forces_i", "expected_forces_j",
                              "expected_forces_k"]),
        ("test_comp_dihedrals", ["expected_energies", "expected_forces_i", "expected_forces_j",
                                 "expected_forces_k", "expected_forces_l"]),
    ):
        for k, v in _ast_arrays(tf, func, names_).items():
            kat[f"{func}/{k}"] = v
    # The same cases evaluated by the reference __plain kernels (the tests' subject)
    indices, bonds, names, molecules, r, CONF = conft.dppc_single()
    cfg = Cfg(); cfg.bonds = list(CONF["bond_2"]); cfg.angle_bonds = list(CONF["bond_3"]); cfg.dihedrals = []
    b2, b3, _, _ = force.prepare_bonds_old(molecules, names, bonds, indices, cfg)
    f = np.zeros_like(r)
    kat["plain/dppc_all_bonds/energy"] = force.compute_bond_forces__plain(f, r.copy(), b2, CONF["L"])
    kat["plain/dppc_all_bonds/f"] = f.copy()
    f = np.zeros_like(r)
    kat["plain/dppc_all_angles/energy"] = force.compute_angle_forces__plain(f, r.copy(), b3, CONF["L"])
    kat["plain/dppc_all_angles/f"] = f.copy()
    indices, bonds, names, molecules, r, CONF = conft.alanine_octapeptide()
    cfg = Cfg(); cfg.bonds = []; cfg.angle_bonds = []; cfg.dihedrals = list(CONF["bond_4"])
    _, _, b4, _ = force.prepare_bonds_old(molecules, names, bonds, indices, cfg)
    f = np.zeros_like(r)
    b4_plain = [(x[0], x[1], x[2], x[3], x[4], x[5]) for x in b4]
    kat["plain/ala_all_dihedrals/energy"] = force.compute_dihedral_forces__plain(f, r.copy(), b4_plain, CONF["L"])
    kat["plain/ala_all_dihedrals/f"] = f.copy()
    np.savez(os.path.join(HERE, "bonded_kat.npz"), **kat)

    # ---------------- Hamiltonians (hymd/hamiltonian.py lambdas) ---------------
    rng = np.random.default_rng(20261203)
    hamg = {}
    Chi = force.Chi
    T = 3
    names3 = ["A", "B", "C"]
    chi_vals = {("A", "B"): 9.6754032616815161, ("A", "C"): -13.2596290315913623,
                ("B", "C"): 0.3852001771213374}
    phi = [rng.uniform(0.0, 2.0, size=(4, 5, 6)) for _ in range(T)]
    for kind in ("SquaredPhi", "DefaultNoChi", "DefaultWithChi"):
        cfg = Cfg()
        cfg.n_types = T
        cfg.n_particles = 123
        cfg.box_size = np.array([4.0, 5.0, 6.0])
        cfg.barostat = "isotropic"          # keep explicit rho0 / a below
        cfg.rho0 = 1.7
        cfg.a = 1.9
        cfg.kappa = 0.05
        cfg.sigma = 0.5
        cfg.self_energy = 0.0
        cfg.type_charges = [0.0] * T
        cfg.coulombtype = None
        cfg.chi = [Chi(atom_1=k[0], atom_2=k[1], interaction_energy=v) for k, v in chi_vals.items()]
        cfg.unique_names = names3
        cfg.type_to_name_map = {i: n for i, n in enumerate(names3)}
        cfg.hamiltonian = kind
        H = ham.get_hamiltonian(cfg)
        hamg[f"{kind}/w0"] = np.asarray(H.w_0(phi), dtype=np.float64)
        for t in range(T):
            hamg[f"{kind}/v_ext{t}"] = np.asarray(H.v_ext[t](phi), dtype=np.float64) * np.ones_like(phi[0])
            hamg[f"{kind}/V_bar_0{t}"] = np.asarray(H.V_bar_0[t](phi), dtype=np.float64) * np.ones_like(phi[0])
        kk = np.array([[0.5321315378106508, -0.6711591309063634, 0.8362051282174443]])
        hamg[f"{kind}/H_k"] = kk
        hamg[f"{kind}/H_v"] = np.array([H.H(kk[0], 0.75)])
    for t in range(T):
        hamg[f"phi{t}"] = phi[t]
    hamg["params"] = np.array([1.7, 1.9, 0.05, 0.5])
    hamg["chi_ab_ac_bc"] = np.array([chi_vals[("A", "B")], chi_vals[("A", "C")], chi_vals[("B", "C")]])
    np.savez(os.path.join(HERE, "hamiltonian.npz"), **hamg)

    # ---------------- misc: dipole redistribution, propensities, integrator ----
    misc = {}
    D = 7
    n = 20
    a = rng.integers(0, n, D); b = rng.integers(0, n, D); c = rng.integers(0, n, D); d = rng.integers(0, n, D)
    fdip = rng.normal(size=(D, 4, 3))
    tm = rng.normal(size=(D, 6, 3, 3))
    dt_ = np.array([1, 0, 1, 1, 2, 1, 0])
    last = np.array([1, 0, 0, 1, 0, 0, 1])
    out = np.zeros((n, 3))
    force.dipole_forces_redistribution(out, fdip, tm, a, b, c, d, dt_, last)
    for k, v in dict(a=a, b=b, c=c, d=d, fdip=fdip, tm=tm, type=dt_, last=last, out=out).items():
        misc[f"dipole_redistribution/{k}"] = v
    for lam in (-1.0, -0.5, 0.0, 0.3, 1.0):
        misc[f"propensity/{lam}"] = force.propensity_potential_coeffs(lam)
    _, _, _, _, positions, velocities, CONF = conft.three_atoms()
    acc = rng.normal(size=velocities.shape)
    misc["integrator/v0"] = velocities
    misc["integrator/r0"] = positions
    misc["integrator/acc"] = acc
    misc["integrator/dt"] = np.array(CONF["dt"])
    misc["integrator/v1"] = integ.integrate_velocity(velocities, acc, CONF["dt"])
    misc["integrator/r1"] = integ.integrate_position(positions, velocities, CONF["dt"])
    ti = os.path.join(ref, "test", "test_integrator.py")
    for k, v in _ast_arrays(ti, "test_integrator_velocity", ["accelerations", "expected_velocities"]).items():
        misc[f"integrator_kat/{k}"] = v
    for k, v in _ast_arrays(ti, "test_integrator_position", ["expected_positions"]).items():
        misc[f"integrator_kat/{k}"] = v
    np.savez(os.path.join(HERE, "misc.npz"), **misc)
    print("wrote golden fixtures to", HERE)


def random_molecules(seed=7, n_mol=60):
    """Seeded random molecules for the topology fixture: 1-16 beads each,
    random trees plus extra edges (rings), names from A-D, molecule ids and
    global indices scrambled, members interleaved in the local order, bond
    rows with -1 anywhere, edges listed from one or both ends, some
    self-bonds.  Returns molecules, names (bytes), bonds (global indices),
    indices, and the term types (plain tuples)."""
    rng = np.random.default_rng(seed)
    alphabet = ["A", "B", "C", "D"]
    sizes = rng.integers(1, 17, n_mol)
    N = int(sizes.sum())
    mol_of = np.repeat(rng.permutation(10 * n_mol)[:n_mol], sizes)
    molecules = mol_of[rng.permutation(N)]
    indices = rng.permutation(N) + 500
    names = np.array([alphabet[x].encode() for x in rng.integers(0, 4, N)])
    rows = [[] for _ in range(N)]
    deg = np.zeros(N, int)

    def link(u, v):
        deg[u] += 1
        deg[v] += 1
        c = rng.integers(0, 3)
        if c != 1:
            rows[u].append(int(indices[v]))
        if c != 0:
            rows[v].append(int(indices[u]))

    for m in np.unique(molecules):
        mem = rng.permutation(np.where(molecules == m)[0])
        for i in range(1, len(mem)):
            cand = [j for j in range(i) if deg[mem[j]] < 4]
            link(mem[i], mem[cand[rng.integers(0, len(cand))]] if cand else mem[i - 1])
        for _ in range(len(mem) // 5):
            u, v = rng.choice(mem, 2, replace=False)
            if deg[u] < 6 and deg[v] < 6:
                link(u, v)
        if len(mem) > 2 and rng.uniform() < 0.2:
            rows[mem[0]].append(int(indices[mem[0]]))
    M = max(len(r) for r in rows) + 1
    bonds = -np.ones((N, M), dtype=np.int64)
    for i, r in enumerate(rows):
        slots = np.sort(rng.permutation(M)[:len(r)])
        bonds[i, slots] = r
    bond_types = [("A", "B", 0.40, 1000.0), ("A", "A", 0.45, 1100.0), ("B", "C", 0.50, 1200.0),
                  ("C", "D", 0.30, 900.0), ("A", "B", 0.41, 800.0), ("D", "A", 0.33, 700.0),
                  ("E", "A", 0.2, 100.0)]
    angle_types = [("A", "B", "C", 120.0, 25.0), ("C", "B", "A", 110.0, 20.0),
                   ("A", "A", "A", 180.0, 30.0), ("B", "C", "D", 100.0, 15.0),
                   ("D", "D", "B", 90.0, 10.0), ("A", "E", "A", 90.0, 10.0)]
    c0 = [[1.0, 2.0, 3.0, 4.0, 5.0], [0.0, 0.0, 0.0, 0.0, 0.0]]
    c1 = [[0.5] * 5, [1.0] * 5, [2.0] * 5, [3.0] * 5]
    dihedral_types = [("A", "B", "C", "D", c0, 0), ("D", "C", "B", "A", c0, 0),
                      ("A", "A", "A", "A", [[1.0] * 5, [0.0, 1.0, 0.0, 1.0, 0.0]], 0),
                      ("A", "B", "A", "B", c1, 1), ("B", "A", "B", "A", c1, 1),
                      ("C", "C", "D", "D", [[2.0] * 5, [0.0] * 5], 2),
                      ("A", "B", "C", "D", [[9.0] * 5, [0.0] * 5], 0),
                      ("B", "B", "A", "C", c0, 0)]
    return molecules, names, bonds, indices, bond_types, angle_types, dihedral_types


def random_topology(ref):
    """topology_random.npz: the reference's prepare_bonds_old / prepare_bonds
    on random_molecules() (inputs, term types and outputs)."""
    _install_stubs()
    pkg = _types.ModuleType("hymd")
    pkg.__path__ = [os.path.join(ref, "hymd")]
    sys.modules["hymd"] = pkg
    logger = _load("hymd.logger", os.path.join(ref, "hymd", "logger.py"), "hymd")
    force = _load("hymd.force", os.path.join(ref, "hymd", "force.py"), "hymd")
    force.Logger = logger.Logger
    molecules, names, bonds, indices, bt, at, dt = random_molecules()

    class Cfg:
        pass
    cfg = Cfg()
    cfg.bonds = [force.Bond(a, b, r0, k) for a, b, r0, k in bt]
    cfg.angle_bonds = [force.Angle(atom_1=a, atom_2=b, atom_3=c, equilibrium=e, strength=k)
                       for a, b, c, e, k in at]
    cfg.dihedrals = [force.Dihedral(atom_1=a, atom_2=b, atom_3=c, atom_4=d, coeffs=co,
                                    dih_type=t) for a, b, c, d, co, t in dt]
    b2, b3, b4, bbi = force.prepare_bonds_old(molecules, names, bonds, indices, cfg)
    packed = force.prepare_bonds(molecules, names, bonds, indices, cfg)
    out = {"molecules": molecules, "names": names, "bonds": bonds, "indices": indices,
           "b4_idx": np.array([[x[0], x[1], x[2], x[3], x[5]] for x in b4],
                              dtype=np.int64).reshape(-1, 5),
           "bb_index": np.asarray(bbi, dtype=np.int64)}
    keys = ["b2a", "b2b", "b2r0", "b2k", "b3a", "b3b", "b3c", "b3t0", "b3k",
            "b4a", "b4b", "b4c", "b4d", "b4coeff", "b4type", "b4last"]
    for k, v in zip(keys, packed):
        out[f"packed/{k}"] = np.asarray(v)
    np.savez(os.path.join(HERE, "topology_random.npz"), **out)
    print("wrote", os.path.join(HERE, "topology_random.npz"), "terms:", len(b2), len(b3),
          len(b4), "bb:", len(bbi))


def reference_root():
    """The HyMD checkout: first command-line argument, else $HYMD_REFERENCE."""
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HYMD_REFERENCE")
    if not ref or not os.path.isdir(os.path.join(ref, "hymd")):
        sys.exit("usage: make_golden.py <HyMD checkout> (or set HYMD_REFERENCE)")
    return ref


if __name__ == "__main__":
    ref = reference_root()
    main(ref)
    random_topology(ref)
