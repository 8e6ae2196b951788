"""Topology preparation on the device (hpf_topology_terms) against the
reference's prepare_bonds output (golden fixtures) and the host restatement:
every packed array bit-exact, same dtypes."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from test_host import PACKED_KEYS, _cfg_for, random_topology_case  # noqa: E402


def _same(a, b):
    return all(x.dtype == y.dtype and x.shape == y.shape and np.array_equal(x, y)
               for x, y in zip(a, b))


def test_random_molecules_match_reference(golden):
    from hymd_gb300.force import prepare_bonds
    t, c = random_topology_case(golden)
    packed = prepare_bonds(t["molecules"], t["names"], t["bonds"], t["indices"], c,
                           device="cuda")
    for k, v in zip(PACKED_KEYS, packed):
        ref = t["packed/" + k]
        assert v.dtype == ref.dtype and np.array_equal(v, ref), k


@pytest.mark.parametrize("fixture", ["dppc_single", "alanine_octapeptide"])
def test_reference_fixtures(golden, fixture):
    from hymd_gb300.force import prepare_bonds
    t = golden("topology.npz")
    p = fixture + "/"
    cfg = _cfg_for(fixture, t)
    packed = prepare_bonds(t[p + "molecules"], t[p + "names"], t[p + "bonds"], t[p + "indices"],
                           cfg, device="cuda")
    for k, v in zip(PACKED_KEYS, packed):
        ref = t[p + "packed/" + k]
        assert v.dtype == ref.dtype and np.array_equal(v, ref), k


def test_molecules_with_solvent(golden):
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
    packed = prepare_bonds(t["mws/molecules"], names, t["mws/bonds"], t["mws/indices"], c,
                           device="cuda")
    for k, v in zip(PACKED_KEYS[:9], packed):
        assert np.array_equal(v, t["mws/packed/" + k]), k
    assert all(len(x) == 0 for x in packed[9:])


@pytest.mark.parametrize("builder", ["homopolymer_melt", "lipid_membrane", "charged_peptides"])
def test_benchmark_systems(builder):
    """Whole-system discovery equals the per-molecule host result tiled over
    the molecules (10k, 162k and 500k beads, the last with CBT dihedrals)."""
    from hymd_gb300 import systems
    from hymd_gb300.force import prepare_bonds
    s = getattr(systems, builder)()
    n = len(s["names"])
    packed = prepare_bonds(s["molecules"], s["names"], s["bonds"], np.arange(n), s["config"],
                           device="cuda")
    assert _same(packed, s["topology"])


def test_host_and_device_agree_with_scrambled_indices(golden):
    """Global indices offset and permuted, molecules in scrambled order."""
    from hymd_gb300.force import prepare_bonds
    t, c = random_topology_case(golden)
    rng = np.random.default_rng(3)
    N = len(t["indices"])
    newid = rng.permutation(N) * 3 + 7
    remap = dict(zip(t["indices"].tolist(), newid.tolist()))
    bonds = np.vectorize(lambda x: remap.get(x, -1))(t["bonds"])
    mol = t["molecules"] * 5 + 11
    host = prepare_bonds(mol, t["names"], bonds, newid, c)
    dev = prepare_bonds(mol, t["names"], bonds, newid, c, device="cuda")
    assert _same(host, dev)


def test_errors_and_empty_input():
    from hymd_gb300 import _lib
    from hymd_gb300.force import Bond, prepare_bonds

    class C:
        pass
    c = C()
    c.bonds = [Bond("A", "A", 0.5, 100.0)]
    c.angle_bonds, c.dihedrals = [], []
    names = np.array([b"A"] * 12)
    # no bonds at all: empty arrays
    packed = prepare_bonds(np.arange(12), names, -np.ones((12, 2), int), np.arange(12), c,
                           device="cuda")
    assert all(len(x) == 0 for x in packed)
    # a partner in another molecule
    bonds = -np.ones((12, 2), int)
    bonds[0, 0] = 7
    mol = np.repeat([0, 1], 6)
    with pytest.raises(_lib.HPFError):
        prepare_bonds(mol, names, bonds, np.arange(12), c, device="cuda")
    # a partner index that no particle has
    bonds[0, 0] = 99
    with pytest.raises(ValueError):
        prepare_bonds(mol, names, bonds, np.arange(12), c, device="cuda")
    # a bead with more than HPF_TOPO_MAX_DEGREE (8) neighbours
    bonds = -np.ones((12, 10), int)
    bonds[0, :10] = np.arange(1, 11)
    with pytest.raises(_lib.HPFError):
        prepare_bonds(np.zeros(12, int), names, bonds, np.arange(12), c, device="cuda")
