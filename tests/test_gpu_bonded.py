"""GPU parity of the bonded kernels against the C restatement of the Fortran
(single-precision variant, the reference's default path) and the FP64 variant."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import bonded as ob  # noqa: E402

FORCE_RTOL = 1e-5
ENERGY_RTOL = 1e-6


def rel_rms(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def peptide_system(seed=0, n_chains=40, n_res=30, box=9.0):
    from hymd_gb300 import systems
    s = systems.charged_peptides(seed=seed, n_chains=n_chains, n_res=n_res,
                                 n_total=n_chains * 2 * n_res + 500, box=box, mesh=16)
    # the random walk puts every bond exactly at r0, where the force is pure
    # rounding; thermal-sized displacements make the comparison meaningful
    rng = np.random.default_rng(seed + 100)
    r = s["positions"] + rng.normal(0.0, 0.05, s["positions"].shape)
    s["positions"] = np.mod(r, s["config"].box()).astype(np.float32)
    return s


def test_bonds_angles_match_oracle():
    from hymd_gb300 import force as gfo
    s = peptide_system(1)
    r = s["positions"]
    box = s["config"].box()
    (b2a, b2b, b2r, b2k, b3a, b3b, b3c, b3t, b3k, *_r) = s["topology"]
    R = torch.as_tensor(r, device="cuda")
    f = torch.zeros_like(R)
    e, pr = gfo.compute_bond_forces(f, R, box, b2a, b2b, b2r, b2k)
    f_ref = np.zeros_like(r)
    e_ref, pr_ref = ob.compute_bond_forces(f_ref, r, box, b2a, b2b, b2r, b2k)
    f64 = np.zeros(r.shape)
    e64, pr64 = ob.compute_bond_forces(f64, r.astype(np.float64), box, b2a, b2b, b2r, b2k,
                                       precision="double")
    assert rel_rms(f.cpu().numpy(), f_ref) < FORCE_RTOL
    assert e == pytest.approx(e_ref, rel=ENERGY_RTOL)
    assert np.allclose(pr, pr64, rtol=1e-5, atol=1e-5 * np.abs(pr64).max())
    fa = torch.zeros_like(R)
    e, pr = gfo.compute_angle_forces(fa, R, box, b3a, b3b, b3c, b3t, b3k)
    fa_ref = np.zeros_like(r)
    e_ref, pr_ref = ob.compute_angle_forces(fa_ref, r, box, b3a, b3b, b3c, b3t, b3k)
    assert rel_rms(fa.cpu().numpy(), fa_ref) < FORCE_RTOL
    assert e == pytest.approx(e_ref, rel=ENERGY_RTOL)


@pytest.mark.parametrize("dipole_flag", [0, 1])
def test_dihedrals_cbt_dipoles_match_oracle(dipole_flag):
    from hymd_gb300 import force as gfo
    s = peptide_system(2)
    r = s["positions"]
    box = s["config"].box()
    (*_h, b4a, b4b, b4c, b4d, coeff, b4t, last) = s["topology"]
    # mix in plain cosine-series (type 0) and improper (type 2) terms
    b4t = b4t.copy()
    b4t[::3] = 0
    b4t[1::7] = 2
    coeff = coeff.copy()
    coeff[1::7, 0, 0] = 0.4
    coeff[1::7, 0, 1] = 30.0
    D = len(b4a)
    R = torch.as_tensor(r, device="cuda")
    f = torch.zeros_like(R)
    dip = torch.zeros((D, 4, 3), device="cuda")
    tm = torch.zeros((D, 6, 3, 3), device="cuda")
    e = gfo.compute_dihedral_forces(f, R, dip, tm, box, b4a, b4b, b4c, b4d, coeff, b4t, last,
                                    dipole_flag)
    f_ref = np.zeros_like(r)
    dip_ref = np.zeros((D, 4, 3), np.float32)
    tm_ref = np.zeros((D, 6, 3, 3), np.float32)
    e_ref = ob.compute_dihedral_forces(f_ref, r, dip_ref, tm_ref, box, b4a, b4b, b4c, b4d, coeff,
                                       b4t, last, dipole_flag)
    assert rel_rms(f.cpu().numpy(), f_ref) < FORCE_RTOL
    assert e == pytest.approx(e_ref, rel=ENERGY_RTOL)
    if dipole_flag:
        assert rel_rms(dip.cpu().numpy(), dip_ref) < 1e-6
        assert rel_rms(tm.cpu().numpy(), tm_ref) < FORCE_RTOL
    else:
        assert not dip.any() and not tm.any()


def test_reference_kat_on_gpu(golden):
    """The reference's own 1e-13 golden vectors (test/test_force.py), held to
    the FP32 bound here; dihedral forces carry the documented sign of the
    production kernel (-grad E)."""
    from hymd_gb300 import force as gfo
    t, k = golden("topology.npz"), golden("bonded_kat.npz")
    r = t["dppc_single/r"].astype(np.float32)
    L = t["dppc_single/L"]
    R = torch.as_tensor(r, device="cuda")
    for i, b in enumerate(t["dppc_single/b2_list"]):
        f = torch.zeros_like(R)
        e, _ = gfo.compute_bond_forces(f, R, L, [int(b[0])], [int(b[1])], [b[2]], [b[3]])
        assert e == pytest.approx(k["test_comp_bonds/expected_energies"][i], rel=1e-4, abs=1e-5)
        assert np.allclose(f.cpu().numpy()[int(b[0])], k["test_comp_bonds/expected_forces_i"][i],
                           rtol=1e-4, atol=1e-3)
    for i, b in enumerate(t["dppc_single/b3_list"]):
        f = torch.zeros_like(R)
        e, _ = gfo.compute_angle_forces(f, R, L, [int(b[0])], [int(b[1])], [int(b[2])], [b[3]],
                                        [b[4]])
        assert e == pytest.approx(k["test_comp_angles/expected_energies"][i], rel=1e-4, abs=1e-5)
    r = t["alanine_octapeptide/r"].astype(np.float32)
    R = torch.as_tensor(r, device="cuda")
    for i, b in enumerate(t["alanine_octapeptide/b4_idx"]):
        f = torch.zeros_like(R)
        coeff = np.zeros((1, 6, 5), np.float32)
        coeff[0, 0] = 1.0
        e = gfo.compute_dihedral_forces(f, R, torch.zeros((1, 4, 3), device="cuda"),
                                        torch.zeros((1, 6, 3, 3), device="cuda"),
                                        t["alanine_octapeptide/L"], [b[0]], [b[1]], [b[2]], [b[3]],
                                        coeff, [b[4]], [0], 0)
        assert e == pytest.approx(k["test_comp_dihedrals/expected_energies"][i], rel=1e-5)
        assert np.allclose(-f.cpu().numpy()[b[0]], k["test_comp_dihedrals/expected_forces_i"][i],
                           rtol=1e-4, atol=1e-4)


def test_dipole_redistribution_matches_reference(golden):
    from hymd_gb300 import force as gfo
    m = golden("misc.npz")
    p = "dipole_redistribution/"
    out = torch.zeros((20, 3), device="cuda")
    gfo.dipole_forces_redistribution(out, m[p + "fdip"], m[p + "tm"], m[p + "a"], m[p + "b"],
                                     m[p + "c"], m[p + "d"], m[p + "type"], m[p + "last"])
    assert np.allclose(out.cpu().numpy(), m[p + "out"], rtol=1e-5, atol=1e-5)


def test_out_of_range_index_is_reported():
    """A bad topology index is a host-visible error, never a device fault."""
    from hymd_gb300 import _lib
    from hymd_gb300 import force as gfo
    R = torch.rand((10, 3), device="cuda")
    f = torch.zeros_like(R)
    with pytest.raises(_lib.HPFError) as ei:
        gfo.compute_bond_forces(f, R, [5.0, 5.0, 5.0], [0, 11], [1, 2], [0.5, 0.5],
                                [100.0, 100.0])
    assert ei.value.code == 4
