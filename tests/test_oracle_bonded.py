"""The bonded oracle (C restatement of cbf/caf/cdf) against the reference's
own known answers (test/test_force.py, 1e-13) and finite differences."""
import numpy as np
import pytest

from oracle import bonded


def test_bonds_match_reference_kat(golden):
    t, k = golden("topology.npz"), golden("bonded_kat.npz")
    r, L = t["dppc_single/r"], t["dppc_single/L"]
    for i, b in enumerate(t["dppc_single/b2_list"]):
        f = np.zeros_like(r)
        e, _ = bonded.compute_bond_forces(f, r, L, [int(b[0])], [int(b[1])], [b[2]], [b[3]],
                                          precision="double")
        assert e == pytest.approx(k["test_comp_bonds/expected_energies"][i], abs=1e-12)
        assert f[int(b[0])] == pytest.approx(k["test_comp_bonds/expected_forces_i"][i], abs=1e-12)
        assert f[int(b[1])] == pytest.approx(k["test_comp_bonds/expected_forces_j"][i], abs=1e-12)


def test_angles_match_reference_kat(golden):
    t, k = golden("topology.npz"), golden("bonded_kat.npz")
    r, L = t["dppc_single/r"], t["dppc_single/L"]
    for i, b in enumerate(t["dppc_single/b3_list"]):
        f = np.zeros_like(r)
        e, _ = bonded.compute_angle_forces(f, r, L, [int(b[0])], [int(b[1])], [int(b[2])],
                                           [b[3]], [b[4]], precision="double")
        assert e == pytest.approx(k["test_comp_angles/expected_energies"][i], abs=1e-12)
        for j, key in enumerate("ijk"):
            assert f[int(b[j])] == pytest.approx(k[f"test_comp_angles/expected_forces_{key}"][i],
                                                 abs=1e-12)


def test_dihedrals_match_reference_kat(golden):
    """Energies equal the KAT; forces equal it with the opposite sign.

    The KAT pins the deprecated Python kernel (hymd/force.py:808-852), whose
    forces are +grad E; the production Fortran cdf (and this oracle) returns
    -grad E, which the finite-difference test below confirms."""
    t, k = golden("topology.npz"), golden("bonded_kat.npz")
    r, L = t["alanine_octapeptide/r"], t["alanine_octapeptide/L"]
    for i, b in enumerate(t["alanine_octapeptide/b4_idx"]):
        f = np.zeros_like(r)
        coeff = np.zeros((1, 6, 5), np.float32)
        coeff[0, 0] = 1.0
        e = bonded.compute_dihedral_forces(
            f, r, np.zeros((1, 4, 3)), np.zeros((1, 6, 3, 3)), L, [b[0]], [b[1]], [b[2]], [b[3]],
            coeff, [b[4]], [0], 0, precision="double")
        assert e == pytest.approx(k["test_comp_dihedrals/expected_energies"][i], abs=1e-12)
        for j, key in enumerate("ijkl"):
            assert -f[b[j]] == pytest.approx(k[f"test_comp_dihedrals/expected_forces_{key}"][i],
                                             abs=1e-12)


def _random_chain_system(seed, n_chain=4, length=8):
    rng = np.random.default_rng(seed)
    L = np.array([6.0, 7.0, 8.0])
    r = []
    for c in range(n_chain):
        p = rng.uniform(0, L)
        for j in range(length):
            r.append(p.copy())
            step = rng.normal(size=3)
            p = p + 0.38 * step / np.linalg.norm(step)
    r = np.mod(np.array(r), L)
    return rng, L, r


@pytest.mark.parametrize("dtype_", [0, 1, 2])
def test_dihedral_forces_are_minus_gradient(dtype_):
    rng, L, r = _random_chain_system(5)
    n = len(r)
    a = np.array([0, 8, 16, 24]); b = a + 1; c = a + 2; d = a + 3
    coeff = np.zeros((4, 6, 5), np.float32)
    coeff[:, 0] = rng.normal(0, 2, size=(4, 5))
    coeff[:, 1] = rng.uniform(-1, 1, size=(4, 5))
    coeff[:, 4] = np.abs(rng.normal(0, 20, size=(4, 5)))
    coeff[:, 5] = rng.uniform(-1, 1, size=(4, 5))
    if dtype_ == 2:
        coeff[:, 0, 0] = 0.3
        coeff[:, 0, 1] = 50.0
    types = np.full(4, dtype_)
    last = np.array([1, 0, 1, 0])

    def energy(rr):
        f = np.zeros_like(rr)
        return bonded.compute_dihedral_forces(
            f, rr, np.zeros((4, 4, 3)), np.zeros((4, 6, 3, 3)), L, a, b, c, d, coeff, types,
            last, 0, precision="double"), f

    _, f = energy(r)
    h = 1e-6
    for atom in np.concatenate([a, b, c, d])[:10]:
        for dd in range(3):
            rp = r.copy(); rp[atom, dd] += h
            rm = r.copy(); rm[atom, dd] -= h
            g = (energy(rp)[0] - energy(rm)[0]) / (2 * h)
            assert -g == pytest.approx(f[atom, dd], rel=1e-5, abs=1e-5)


def test_single_and_double_variants_agree():
    rng, L, r = _random_chain_system(7)
    a = np.arange(0, 31); a = a[(a % 8) < 7]; b = a + 1
    r0 = np.full(len(a), 0.47); k = np.full(len(a), 1250.0)
    f32 = np.zeros((len(r), 3), np.float32)
    f64 = np.zeros((len(r), 3))
    e32, p32 = bonded.compute_bond_forces(f32, r.astype(np.float32), L, a, b, r0, k)
    e64, p64 = bonded.compute_bond_forces(f64, r, L, a, b, r0, k, precision="double")
    assert e32 == pytest.approx(e64, rel=1e-5)
    assert np.allclose(f32, f64, rtol=1e-4, atol=1e-3)
