"""Host-side logic (no GPU): the C-ABI library, topology preparation,
functional extraction, and the synthetic workloads."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def built_lib():
    from hymd_gb300 import build
    return build.build()


def test_library_exports_every_declared_symbol(built_lib):
    import ctypes
    from hymd_gb300 import _lib
    L = ctypes.CDLL(built_lib)
    names = _lib.header_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    # every declared entry point has a ctypes signature
    assert set(names) - {"hpf_status_string"} == set(_lib._SIGNATURES)
    L.hpf_status_string.restype = ctypes.c_char_p
    assert L.hpf_status_string(4) == b"HPF_ERR_INDEX"


def _cfg_for(fixture, t):
    from hymd_gb300.force import Angle, Bond, Dihedral

    class C:
        pass
    c = C()
    if fixture == "dppc_single":
        c.bonds = [Bond("N", "P", 0.47, 1250.0), Bond("P", "G", 0.47, 1250.0),
                   Bond("G", "G", 0.37, 1250.0), Bond("G", "C", 0.47, 1250.0),
                   Bond("C", "C", 0.47, 1250.0)]
        c.angle_bonds = [Angle(atom_1=a, atom_2=b, atom_3=cc, equilibrium=e, strength=25.0)
                         for a, b, cc, e in (("P", "G", "G", 120.0), ("P", "G", "C", 180.0),
                                             ("G", "C", "C", 180.0), ("C", "C", "C", 180.0))]
        c.dihedrals = []
    else:
        c.bonds = [Bond("BB", "SC", 0.27, 100000), Bond("BB", "BB", 0.35, 4000)]
        c.angle_bonds = [Angle(atom_1="BB", atom_2="BB", atom_3="BB", equilibrium=127,
                               strength=20),
                         Angle(atom_1="BB", atom_2="BB", atom_3="SC", equilibrium=100,
                               strength=25)]
        c.dihedrals = [Dihedral("BB", "BB", "BB", "BB",
                                np.array([[1, 1, 1, 1, 1], [0, 0, 0, 0, 0]]), 0)]
    return c


@pytest.mark.parametrize("fixture", ["dppc_single", "alanine_octapeptide"])
def test_prepare_bonds_bit_exact_with_reference(golden, fixture):
    from hymd_gb300.force import prepare_bonds, prepare_bonds_old
    t = golden("topology.npz")
    p = fixture + "/"
    cfg = _cfg_for(fixture, t)
    b2, b3, b4, bbi = prepare_bonds_old(t[p + "molecules"], t[p + "names"], t[p + "bonds"],
                                        t[p + "indices"], cfg)
    assert np.array_equal(np.array(b2, dtype=np.float64).reshape(-1, 4), t[p + "b2_list"])
    assert np.array_equal(np.array(b3, dtype=np.float64).reshape(-1, 5), t[p + "b3_list"])
    assert np.array_equal(np.array([[x[0], x[1], x[2], x[3], x[5]] for x in b4],
                                   dtype=np.int64).reshape(-1, 5), t[p + "b4_idx"])
    assert np.array_equal(np.asarray(bbi, dtype=np.int64), t[p + "bb_index"])
    packed = prepare_bonds(t[p + "molecules"], t[p + "names"], t[p + "bonds"], t[p + "indices"],
                           cfg)
    keys = ["b2a", "b2b", "b2r0", "b2k", "b3a", "b3b", "b3c", "b3t0", "b3k",
            "b4a", "b4b", "b4c", "b4d", "b4coeff", "b4type", "b4last"]
    for k, v in zip(keys, packed):
        ref = t[p + "packed/" + k]
        assert v.dtype == ref.dtype and np.array_equal(v, ref), k


def test_prepare_bonds_molecules_with_solvent(golden):
    from hymd_gb300.force import Angle, Bond, prepare_bonds
    t = golden("topology.npz")
    names = t["mws/names"]
    uniq = sorted(set(n.decode() for n in names))

    class C:
        pass
    c = C()
    c.bonds = [Bond(x, y, 0.5, 1000.0) for i, x in enumerate(uniq) for y in uniq[i:]]
    c.angle_bonds = [Angle(atom_1=x, atom_2=y, atom_3=z, equilibrium=120.0, strength=25.0)
                     for x in uniq for y in uniq for z in uniq if x <= z]
    c.dihedrals = []
    packed = prepare_bonds(t["mws/molecules"], names, t["mws/bonds"], t["mws/indices"], c)
    for k, v in zip(["b2a", "b2b", "b2r0", "b2k", "b3a", "b3b", "b3c", "b3t0", "b3k"], packed):
        assert np.array_equal(v, t["mws/packed/" + k]), k


def random_topology_case(golden):
    """Inputs and reference outputs of topology_random.npz, with the term
    types rebuilt (as this package's dataclasses) from the generator."""
    import importlib.util
    import os
    from hymd_gb300.force import Angle, Bond, Dihedral
    path = os.path.join(os.path.dirname(__file__), "golden", "make_golden.py")
    spec = importlib.util.spec_from_file_location("make_golden", path)
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    molecules, names, bonds, indices, bt, at, dt = mg.random_molecules()
    t = golden("topology_random.npz")
    for k, v in (("molecules", molecules), ("names", names), ("bonds", bonds),
                 ("indices", indices)):
        assert np.array_equal(t[k], v), k

    class C:
        pass
    c = C()
    c.bonds = [Bond(a, b, r0, k) for a, b, r0, k in bt]
    c.angle_bonds = [Angle(atom_1=a, atom_2=b, atom_3=x, equilibrium=e, strength=k)
                     for a, b, x, e, k in at]
    c.dihedrals = [Dihedral(a, b, x, d, co, ty) for a, b, x, d, co, ty in dt]
    return t, c


PACKED_KEYS = ["b2a", "b2b", "b2r0", "b2k", "b3a", "b3b", "b3c", "b3t0", "b3k",
               "b4a", "b4b", "b4c", "b4d", "b4coeff", "b4type", "b4last"]


def test_prepare_bonds_random_molecules_bit_exact_with_reference(golden):
    """Branched and ring molecules with scrambled ids, duplicate, reversed and
    equal-coefficient term types: the packed arrays equal the reference's."""
    from hymd_gb300.force import prepare_bonds, prepare_bonds_old
    t, c = random_topology_case(golden)
    _, _, b4, bbi = prepare_bonds_old(t["molecules"], t["names"], t["bonds"], t["indices"], c)
    assert np.array_equal(np.array([[x[0], x[1], x[2], x[3], x[5]] for x in b4],
                                   dtype=np.int64).reshape(-1, 5), t["b4_idx"])
    assert np.array_equal(np.asarray(bbi, dtype=np.int64), t["bb_index"])
    packed = prepare_bonds(t["molecules"], t["names"], t["bonds"], t["indices"], c)
    for k, v in zip(PACKED_KEYS, packed):
        ref = t["packed/" + k]
        assert v.dtype == ref.dtype and np.array_equal(v, ref), k


def test_traversal_order_matches_networkx_on_random_graphs():
    nx = pytest.importorskip("networkx")
    from hymd_gb300.force import _bfs_paths, _simple_paths
    rng = np.random.default_rng(0)
    for trial in range(20):
        n = 12
        G = nx.Graph()
        adj = {}
        for u in rng.permutation(n):
            G.add_node(int(u))
            adj.setdefault(int(u), {})
            for v in rng.integers(0, n, 2):
                if v != u:
                    G.add_edge(int(u), int(v))
                    adj.setdefault(int(v), {})
                    adj[int(u)].setdefault(int(v), None)
                    adj[int(v)].setdefault(int(u), None)
        adj = {k: list(v) for k, v in adj.items()}
        assert list(G.nodes()) == list(adj)
        for s in G.nodes():
            ref = nx.single_source_shortest_path(G, s)
            mine = _bfs_paths(adj, s)
            assert list(ref.items()) == list(mine.items())


def test_propensity_and_index_topology(golden):
    from hymd_gb300.force import propensity_potential_coeffs
    m = golden("misc.npz")
    for lam in (-1.0, -0.5, 0.0, 0.3, 1.0):
        assert np.array_equal(propensity_potential_coeffs(lam), m[f"propensity/{lam}"])


def test_quadratic_forms_match_reference_lambdas(golden):
    from hymd_gb300.config import Config
    from hymd_gb300.force import Chi
    from hymd_gb300.hamiltonian import get_hamiltonian, quadratic_form
    g = golden("hamiltonian.npz")
    rho0, a, kappa, sigma = g["params"]
    ab, ac, bc = g["chi_ab_ac_bc"]
    phi = [g["phi0"], g["phi1"], g["phi2"]]
    for kind in ("SquaredPhi", "DefaultNoChi", "DefaultWithChi"):
        cfg = Config(n_steps=1, time_step=0.01, mesh_size=8, sigma=sigma, kappa=kappa,
                     box_size=[4.0, 5.0, 6.0], n_particles=123, n_types=3, barostat="isotropic",
                     rho0=rho0, a=a, hamiltonian=kind, unique_names=["A", "B", "C"],
                     type_to_name_map={0: "A", 1: "B", 2: "C"},
                     chi=[Chi("A", "B", ab), Chi("A", "C", ac), Chi("B", "C", bc)])
        h = get_hamiltonian(cfg)
        assert np.allclose(h.w_0(phi), g[kind + "/w0"], rtol=1e-13, atol=1e-12)
        for t in range(3):
            assert np.allclose(h.v_ext[t](phi), g[f"{kind}/v_ext{t}"], rtol=1e-13, atol=1e-12)
        Q, b, c, s = quadratic_form(h)

        class Foreign:  # a reference-style object: only w_0 and config
            config = cfg
            w_0 = staticmethod(h.w_0)
        Q2, b2, c2, _ = quadratic_form(Foreign(), 3)
        assert np.allclose(Q, Q2, rtol=1e-9, atol=1e-9)
        assert np.allclose(b, b2, rtol=1e-9, atol=1e-7)
        assert c == pytest.approx(c2, rel=1e-9)


def test_non_quadratic_functional_is_rejected():
    from hymd_gb300.config import Config
    from hymd_gb300.hamiltonian import quadratic_form
    cfg = Config(n_steps=1, time_step=0.01, mesh_size=8, sigma=0.5, kappa=0.1, n_types=2)

    class Cubic:
        config = cfg

        @staticmethod
        def w_0(phi):
            return phi[0] ** 3 + phi[1]

    with pytest.raises(NotImplementedError):
        quadratic_form(Cubic(), 2)


def test_synthetic_workloads_shapes():
    from hymd_gb300 import systems
    s = systems.lipid_membrane()
    assert s["positions"].shape == (162000, 3)
    assert len(s["topology"][0]) == 66000 and len(s["topology"][4]) == 48000
    assert np.all((s["positions"] >= 0) & (s["positions"] < 27.0))
    s = systems.homopolymer_melt()
    assert s["positions"].shape == (10000, 3) and len(s["topology"][0]) == 9000


def test_integrator_formula_matches_reference_kat(golden):
    """The velocity-Verlet pieces used by oracle/md.py against the known answers
    of the reference's test/test_integrator.py."""
    m = golden("misc.npz")
    dt = float(m["integrator/dt"])
    v0, r0 = m["integrator/v0"], m["integrator/r0"]
    acc = m["integrator_kat/accelerations"]
    np.testing.assert_allclose(v0 + 0.5 * dt * acc, m["integrator_kat/expected_velocities"],
                               rtol=0, atol=1e-13)
    np.testing.assert_allclose(r0 + dt * v0, m["integrator_kat/expected_positions"], rtol=0,
                               atol=1e-13)


def test_adjoint_functional_coefficients_match_oracle():
    """The (Q, b, c) the adjoint differentiates are those of the three
    reference functionals (oracle/hamiltonian.py restates hymd/hamiltonian.py)."""
    from hymd_gb300.adjoint import functional_coefficients
    from oracle import hamiltonian as oh
    rng = np.random.default_rng(1)
    T = 4
    chi = rng.uniform(0, 20, (T, T))
    chi = 0.5 * (chi + chi.T)
    for kind in ("DefaultWithChi", "DefaultNoChi", "SquaredPhi"):
        Q, b, c = functional_coefficients(kind, chi, 0.05, 8.3, 8.0)
        ref = oh.quadratic_from_params(kind, T, 0.05, 8.3, 8.0, chi)
        assert np.allclose(Q, ref.Q, rtol=1e-14) and np.allclose(b, ref.b, rtol=1e-14)
        assert c == pytest.approx(ref.c, rel=1e-14)


def test_ctypes_signatures_match_header_parameter_counts():
    """Every ctypes binding in _lib._SIGNATURES has as many parameters as its
    declaration in include/hpf_gb300.h (a binding that drifts from the
    header would pass the wrong arguments without any other symptom)."""
    import re
    from hymd_gb300 import _lib
    txt = open(_lib.HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    decls = {}
    for m in re.finditer(r"^(?:int|int64_t|const char\*)\s+(hpf_\w+)\s*\(([^;]*?)\)\s*;", txt,
                         re.M | re.S):
        params = m.group(2).strip()
        n = 0 if params in ("", "void") else len(params.split(","))
        decls[m.group(1)] = n
    assert set(_lib._SIGNATURES) <= set(decls)
    bad = {k: (len(v), decls[k]) for k, v in _lib._SIGNATURES.items() if len(v) != decls[k]}
    assert not bad, bad
