"""GPU rRESPA steps against the oracle loop, and graph replay against eager."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import hamiltonian as oh  # noqa: E402
from oracle import md as omd  # noqa: E402


def rel_rms(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def _melt():
    from hymd_gb300 import systems
    s = systems.homopolymer_melt(seed=11, n_chains=300, length=10, box=6.0, mesh=24)
    cfg = s["config"]
    from hymd_gb300.hamiltonian import get_hamiltonian
    ham = get_hamiltonian(cfg)
    fun = oh.quadratic_from_params("DefaultWithChi", 2, cfg.kappa, cfg.rho0, cfg.a,
                                   np.array([[0, 15.0], [15.0, 0]]))
    return s, cfg, ham, fun


def test_respa_step_matches_oracle():
    from hymd_gb300.md import RespaMD
    s, cfg, ham, fun = _melt()
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    md.prime()
    r = s["positions"].copy()
    v = s["velocities"].copy()
    ff = omd.field_forces(r, s["types"], cfg, fun)
    assert rel_rms(md.f_field.cpu().numpy(), ff) < 1e-5
    for _ in range(2):
        md.step()
        r, v, ff = omd.respa_step(r, v, ff, s["types"], s["topology"], cfg, fun)
    rg = md.r.cpu().numpy()
    d = np.abs(rg - r)
    d = np.minimum(d, cfg.box()[None, :] - d)  # wrapped coordinates
    assert np.sqrt(np.mean(d ** 2)) < 1e-5 * np.sqrt(np.mean(r ** 2))
    assert rel_rms(md.v.cpu().numpy(), v) < 1e-4
    assert rel_rms(md.f_field.cpu().numpy(), ff) < 1e-4
    md.check_errors()


def test_graph_replay_matches_eager():
    from hymd_gb300.md import RespaMD
    s, cfg, ham, fun = _melt()
    a = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    b = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    for m in (a, b):
        m.prime()
    a.capture()  # capture() runs one warm-up step eagerly
    b.step()
    a.run(3)
    for _ in range(3):
        b.step()
    torch.cuda.synchronize()
    assert rel_rms(a.r.cpu().numpy(), b.r.cpu().numpy()) < 1e-6
    assert rel_rms(a.v.cpu().numpy(), b.v.cpu().numpy()) < 1e-5


@pytest.mark.parametrize("n_res,max_block_beads", [(40, 256), (40, 36), (10, 36)])
def test_fused_inner_loop_matches_per_term_path(n_res, max_block_beads):
    """Molecule-blocked fused kernel vs the per-term launch sequence on a
    peptide system with CBT dihedrals, dipoles and PIC electrostatics: chains
    of 80 beads (one CTA per group, groups of 3 or 1 chains) and of 20 beads
    (one warp per group of 36 beads at most)."""
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    s = systems.charged_peptides(seed=7, n_chains=30, n_res=n_res, n_total=6000, box=8.0,
                                 mesh=32)
    cfg = s["config"]
    ham = get_hamiltonian(cfg)
    kw = dict(topology=s["topology"], charges=s["charges"])
    a = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, fused=True,
                max_block_beads=max_block_beads, **kw)
    b = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, fused=False, **kw)
    assert a.plan is not None and b.plan is None
    info = a.plan_info()
    per = 2 * n_res
    assert info["free_beads"] == 6000 - 30 * per
    assert info["max_block_beads"] <= max(max_block_beads, per)
    assert info["mol_blocks"] >= 30 * per // max(max_block_beads, per)
    for m in (a, b):
        m.prime()
        m.run(2)
    torch.cuda.synchronize()
    assert rel_rms(a.r.cpu().numpy(), b.r.cpu().numpy()) < 1e-6
    assert rel_rms(a.v.cpu().numpy(), b.v.cpu().numpy()) < 1e-5
    assert rel_rms(a.dipoles.cpu().numpy(), b.dipoles.cpu().numpy()) < 1e-5
    assert rel_rms(a.transfer.cpu().numpy(), b.transfer.cpu().numpy()) < 1e-4
    ea, eb = a.energies(), b.energies()
    for x, y in zip(ea, eb):
        assert x == pytest.approx(y, rel=1e-5)
    a.check_errors()
    b.check_errors()


def test_integrator_matches_reference_kat(golden):
    """integrate_velocity / integrate_position against the known answers of the
    reference's test/test_integrator.py (three_atoms fixture), at FP32."""
    from hymd_gb300.integrator import integrate_position, integrate_velocity
    m = golden("misc.npz")
    dt = float(m["integrator/dt"])
    v0 = torch.tensor(m["integrator/v0"], dtype=torch.float32, device="cuda")
    r0 = torch.tensor(m["integrator/r0"], dtype=torch.float32, device="cuda")
    acc = torch.tensor(m["integrator_kat/accelerations"], dtype=torch.float32, device="cuda")
    v1 = integrate_velocity(v0, acc, dt)
    r1 = integrate_position(r0, v0, dt)
    torch.cuda.synchronize()
    np.testing.assert_allclose(v1.cpu().numpy(), m["integrator_kat/expected_velocities"],
                               rtol=2e-6, atol=1e-6)
    np.testing.assert_allclose(r1.cpu().numpy(), m["integrator_kat/expected_positions"],
                               rtol=2e-6, atol=1e-6)
    # the inputs are not changed in place (hymd/integrator.py:9-73 returns new arrays)
    assert torch.equal(v0.cpu(), torch.tensor(m["integrator/v0"], dtype=torch.float32))
    # within one FP32 rounding of the reference's expressions evaluated in FP32
    v0n = m["integrator/v0"].astype(np.float32)
    an = m["integrator_kat/accelerations"].astype(np.float32)
    want_v = v0n + np.float32(0.5 * dt) * an
    want_r = m["integrator/r0"].astype(np.float32) + np.float32(dt) * v0n
    assert np.all(np.abs(v1.cpu().numpy() - want_v) <= 2 * np.spacing(np.abs(want_v)))
    assert np.all(np.abs(r1.cpu().numpy() - want_r) <= 2 * np.spacing(np.abs(want_r)))


def test_plan_forces_match_per_term_kernels_and_are_reproducible():
    """hpf_respa_forces (the fused plan's deterministic gather, no
    integration) against the per-term drop-in kernels (atomics) on a peptide
    system with CBT dihedrals: same forces to FP32 rounding, same energies,
    and bit-identical on repeated calls."""
    from hymd_gb300 import _lib, systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    s = systems.charged_peptides(seed=9, n_chains=20, n_res=30, n_total=3000, box=7.0, mesh=24)
    cfg = s["config"]
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, get_hamiltonian(cfg),
                 topology=s["topology"], max_block_beads=36)
    st = _lib.stream_ptr()
    md._bonded(st, 0)
    ref = (md.f_bond + md.f_angle + md.f_dih).cpu().numpy()
    outs = []
    for _ in range(2):
        f = torch.zeros_like(md.r)
        out = torch.zeros(10, dtype=torch.float64, device="cuda")
        _lib.call("hpf_respa_forces", md.plan, _lib.ptr(md.r), _lib.ptr(f), _lib.ptr(md.box),
                  _lib.ptr(out), _lib.ptr(md.err), st)
        outs.append((f.clone(), out.cpu().numpy()))
    assert torch.equal(outs[0][0], outs[1][0])
    got, e = outs[0][0].cpu().numpy(), outs[0][1]
    assert rel_rms(got, ref) < 1e-6
    for k, ws in ((0, md.ws_bond), (4, md.ws_angle), (8, md.ws_dih)):
        assert e[k] == pytest.approx(float(ws[0].item()), rel=1e-5)
    md.check_errors()


@pytest.mark.parametrize("thermostat", [False, True])
def test_sorted_bead_order_gives_the_same_trajectory(thermostat):
    """sort_particles() only changes the memory order: a sorted run, read back
    in the caller's order, follows the unsorted run (bit for bit without the
    thermostat, whose sums then run in another order; to FP32 rounding with
    it)."""
    from hymd_gb300.md import RespaMD
    s, cfg, ham, fun = _melt()
    a = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    b = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    perm = b.sort_particles()
    assert not torch.equal(perm, torch.arange(len(perm), device=perm.device))
    for m in (a, b):
        if thermostat:
            m.couple(thermostat=True, seed=4, n_steps=20)
        m.prime()
        m.run(3)
    torch.cuda.synchronize()
    rb, vb = b.in_input_order(b.r), b.in_input_order(b.v)
    if thermostat:
        assert rel_rms(rb.cpu().numpy(), a.r.cpu().numpy()) < 1e-6
        assert rel_rms(vb.cpu().numpy(), a.v.cpu().numpy()) < 1e-5
    else:
        assert torch.equal(rb, a.r) and torch.equal(vb, a.v)
    a.check_errors()
    b.check_errors()


def test_run_host_matches_device_resident_steps():
    """RespaMD.run_host (state copied in from page-locked host tensors, the
    captured step, positions copied out) equals the device-resident replay."""
    from hymd_gb300.md import RespaMD
    s, cfg, ham, fun = _melt()
    a = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    b = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    for m in (a, b):
        m.prime()
        m.capture()
    torch.cuda.synchronize()
    r_h = a.r.cpu().pin_memory()
    v_h = a.v.cpu().pin_memory()
    r_out = torch.empty_like(r_h).pin_memory()
    a.run_host(r_h, v_h, r_out)
    b.run(1)
    torch.cuda.synchronize()
    assert torch.equal(r_out, a.r.cpu())
    assert torch.equal(r_out, b.r.cpu())
    assert torch.equal(a.v, b.v)
    with pytest.raises(ValueError):
        a.run_host(r_h.clone(), v_h, r_out)  # not page-locked
    a.check_errors()


@pytest.mark.parametrize("path", ["fused", "cufft"])
def test_pic_step_on_charged_list_matches_full_pic_step(path):
    """hpf_pic_step_list over the charged beads gives the full step's forces
    bit for bit (fixed-point paint: the q = 0 beads add nothing) and leaves
    the other rows untouched; an index out of range is flagged."""
    from hymd_gb300 import _lib
    from hymd_gb300.field import ParticleMesh
    rng = np.random.default_rng(21)
    n, box = 20000, np.array([7.0, 7.5, 8.0])
    r = torch.as_tensor((rng.uniform(0, 1, (n, 3)) * box).astype(np.float32), device="cuda")
    q = np.zeros(n, np.float32)
    sel = rng.permutation(n)[:900]
    q[sel] = rng.choice([-1.0, 1.0], 900).astype(np.float32)
    Q = torch.as_tensor(q, device="cuda")
    idx = torch.as_tensor(np.sort(sel).astype(np.int32), device="cuda")
    pm = ParticleMesh((32, 32, 32), box, 2)
    _lib.call("hpf_ctx_set_functional", pm._h, _lib.dvec(np.zeros(4)), _lib.dvec(np.zeros(2)),
              0.0, 0.5)
    pm.spectral = path
    fa = torch.zeros_like(r)
    fb = torch.full_like(r, 7.0)
    sa, sb = _lib.new_workspace(r.device), _lib.new_workspace(r.device)
    _lib.call("hpf_pic_step", pm._h, _lib.ptr(r), _lib.ptr(Q), n, 1.7, _lib.ptr(fa), None, None,
              None, None, _lib.ptr(sa), None, _lib.stream_ptr())
    _lib.call("hpf_pic_step_list", pm._h, _lib.ptr(r), _lib.ptr(Q), _lib.ptr(idx), idx.numel(), n,
              1.7, _lib.ptr(fb), _lib.ptr(sb), None, _lib.stream_ptr())
    torch.cuda.synchronize()
    mask = torch.zeros(n, dtype=torch.bool, device="cuda")
    mask[idx.long()] = True
    assert torch.equal(fb[mask], fa[mask])
    assert torch.all(fb[~mask] == 7.0)
    assert torch.equal(sa[:1], sb[:1])
    pm.check_errors()
    bad = idx.clone()
    bad[3] = n
    _lib.call("hpf_pic_step_list", pm._h, _lib.ptr(r), _lib.ptr(Q), _lib.ptr(bad), bad.numel(), n,
              1.7, _lib.ptr(fb), None, None, _lib.stream_ptr())
    with pytest.raises(_lib.HPFError):
        pm.check_errors()


def test_md_with_charges_compact_pic_matches_full_pic():
    """The MD loop's PIC step with the charge paint over the charged beads
    against the full hpf_pic_step: bit-identical forces and trajectories
    (deterministic paint; the same readout and kick)."""
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    s = systems.charged_peptides(seed=9, n_chains=20, n_res=20, n_total=8000, box=9.0, mesh=32)
    cfg = s["config"]
    ham = get_hamiltonian(cfg)
    kw = dict(topology=s["topology"], charges=s["charges"])
    a = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, **kw)
    b = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, **kw)
    from hymd_gb300 import _lib

    def full_field(st, sums=None, pos_scale=None, kick=None, painted=False):
        assert not painted
        _lib.call("hpf_field_step", b.pm._h, _lib.ptr(b.r), _lib.ptr(b.types), b.n, b.masses,
                  _lib.ptr(b.f_field), _lib.ptr(sums),
                  None if pos_scale is None else _lib.ctypes.c_void_p(pos_scale), None, st)
        _lib.call("hpf_pic_step", b.pm._h, _lib.ptr(b.r), _lib.ptr(b.charges), b.n,
                  float(b.elec_factor), _lib.ptr(b.f_elec), None, None, None, None, None, kick,
                  st)
    b._field = full_field
    b.FUSE_PAINT = False  # the full PIC step paints every bead itself
    for m in (a, b):
        m.couple(thermostat=True, seed=3, n_steps=20)
        m.prime()
    torch.cuda.synchronize()
    assert a.charged.numel() == int(np.count_nonzero(s["charges"]))
    assert torch.equal(a.f_elec, b.f_elec)
    for m in (a, b):
        m.capture()
        m.run(3)
    torch.cuda.synchronize()
    assert torch.equal(a.r, b.r) and torch.equal(a.v, b.v)
    a.check_errors()
    b.check_errors()


@pytest.mark.parametrize("captured", [False, True])
def test_resort_keeps_trajectory(captured):
    """RespaMD.resort() between steps (the beads re-sorted by mesh cell in
    place, the plan's bead lists, the bonded indices and the charged-bead
    list remapped on the device): in NVE every per-bead result is independent
    of the memory order, so positions and velocities in the caller's order
    equal those of the run without re-sorting, bit for bit -- also when the
    step was captured in graphs before the re-sorts."""
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    s = systems.charged_peptides(seed=5, n_chains=12, n_res=30, n_total=6000, box=8.0, mesh=32)
    cfg = s["config"]
    ham = get_hamiltonian(cfg)
    kw = dict(topology=s["topology"], charges=s["charges"])
    a = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, **kw)
    b = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, **kw)
    for m in (a, b):
        m.prime()
        if captured:
            m.capture()
    a.resort_every = 2
    a.run(6)
    b.run(6)
    torch.cuda.synchronize()
    assert a.resorts == 3 and a.perm is not None
    assert torch.equal(a.in_input_order(a.r), b.r)
    assert torch.equal(a.in_input_order(a.v), b.v)
    assert torch.equal(a.in_input_order(a.f_elec), b.f_elec)
    a.check_errors()
    b.check_errors()
    # the lists handed back in memory order: charged and free beads ascending,
    # each molecule in one stretch of memory
    ch = a.charged.long()
    assert torch.all(ch[1:] > ch[:-1])
    assert torch.equal(ch, torch.nonzero(a.charges != 0).reshape(-1))
    fr = a._free_ids.long()
    assert fr.numel() and torch.all(fr[1:] > fr[:-1])
    mol = a._mol.long()
    first = torch.full((a.n,), a.n, dtype=torch.long, device=mol.device)
    last = torch.full((a.n,), -1, dtype=torch.long, device=mol.device)
    idx = torch.arange(a.n, device=mol.device)
    first.scatter_reduce_(0, mol, idx, "amin")
    last.scatter_reduce_(0, mol, idx, "amax")
    size = torch.bincount(mol, minlength=a.n)
    used = size > 0
    assert torch.equal((last - first + 1)[used], size[used])
    assert int(size.max()) == 60  # the 30-residue chains (60 beads) are whole molecules


def test_bead_sort_order_keeps_trajectory():
    """The "bead" sort order (every bead by its own cell) gives the same
    trajectory in the caller's order as the unsorted run."""
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    s = systems.charged_peptides(seed=6, n_chains=8, n_res=20, n_total=4000, box=7.0, mesh=28)
    cfg = s["config"]
    ham = get_hamiltonian(cfg)
    kw = dict(topology=s["topology"], charges=s["charges"])
    a = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, **kw)
    b = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, **kw)
    a.sort_particles(order="bead")
    for m in (a, b):
        m.prime()
        m.capture()
    a.resort_every = 3
    a.run(6)
    b.run(6)
    torch.cuda.synchronize()
    assert a.resorts == 2
    assert torch.equal(a.in_input_order(a.r), b.r)
    assert torch.equal(a.in_input_order(a.v), b.v)
    a.check_errors()


@pytest.mark.parametrize("barostat", [None, "isotropic"])
def test_concurrent_charge_chain_matches_sequential(barostat):
    """hpf_field_pic_step (the charge chain of the field step on a second
    stream beside the density chain, joined before the charge readout and
    kick) against hpf_field_step followed by hpf_pic_step_list on one stream:
    the same kernels on separate scratch, so positions, velocities and both
    force arrays are bit-identical after captured NVT (CSVR) steps, also when
    the barostat rescales the positions in the density paint."""
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    s = systems.charged_peptides(seed=8, n_chains=10, n_res=25, n_total=5000, box=7.5, mesh=32)
    cfg = s["config"]
    cfg.tau_p, cfg.n_b = 1.0, 1
    ham = get_hamiltonian(cfg)
    kw = dict(topology=s["topology"], charges=s["charges"])
    a = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, **kw)
    b = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, **kw)
    b.CONCURRENT_PIC = False
    # the paint stays separate on both (with the barostat a fused paint
    # agrees with it to rounding only; tested below)
    a.FUSE_PAINT = b.FUSE_PAINT = False
    assert a.pm.spectral == "fused"
    for m in (a, b):
        m.couple(thermostat=True, barostat=barostat, seed=9, n_steps=20)
        m.prime()
        m.capture()
        m.run(5)
    torch.cuda.synchronize()
    for name in ("r", "v", "f_field", "f_elec"):
        assert torch.equal(getattr(a, name), getattr(b, name)), name
    assert torch.equal(a.box, b.box)
    a.check_errors()
    b.check_errors()


@pytest.mark.parametrize("kind", ["peptide_cta", "peptide_warp", "melt"])
def test_paint_fused_into_respa_matches_separate_paint(kind):
    """hpf_respa_step_paint (each bead deposited on the mesh by the rRESPA
    kernel where it leaves its final position) followed by the field step
    with painted = 1, against the separate paint: the int64 fixed-point
    accumulators are order-independent, so after captured NVT (CSVR) steps
    positions, velocities and field forces are bit-identical -- for chains in
    CTA groups and in warp groups, with and without the charge grid."""
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    if kind == "melt":
        s = systems.homopolymer_melt(seed=12, n_chains=300, length=10, box=6.0, mesh=24)
        kw = dict(topology=s["topology"])
    else:
        n_res = 40 if kind == "peptide_cta" else 10
        s = systems.charged_peptides(seed=13, n_chains=12, n_res=n_res, n_total=5000, box=7.5,
                                     mesh=32)
        kw = dict(topology=s["topology"], charges=s["charges"])
    cfg = s["config"]
    ham = get_hamiltonian(cfg)
    a = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, **kw)
    b = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, **kw)
    b.FUSE_PAINT = False
    assert a.plan is not None and a.pm.spectral == "fused"
    for m in (a, b):
        m.couple(thermostat=True, seed=10, n_steps=20)
        m.prime()
    assert a._paint_fused and not b._paint_fused
    a.step()
    b.step()
    for m in (a, b):
        m.capture()
        m.run(4)
    torch.cuda.synchronize()
    names = ["r", "v", "f_field"] + (["f_elec"] if kind != "melt" else [])
    for name in names:
        assert torch.equal(getattr(a, name), getattr(b, name)), name
    a.check_errors()
    b.check_errors()


def test_paint_fused_with_isotropic_barostat_matches_separate_paint():
    """With the isotropic SCR barostat the fused paint deposits the unscaled
    positions into the old box (grid coordinates r n / L unchanged by
    r -> alpha r, L -> alpha L) and the positions are scaled afterwards;
    against the separate paint of the scaled positions the deposits differ
    only by FP32 rounding of the coordinates, so after captured NPT (CSVR +
    SCR) steps positions, velocities, forces and box agree to that level."""
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    s = systems.lipid_membrane(seed=9, n_lipids=60, n_water=900, box=5.6, mesh=24)
    cfg = s["config"]
    cfg.tau_p, cfg.n_b = 1.0, 1
    ham = get_hamiltonian(cfg)
    a = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    b = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    b.FUSE_PAINT = False
    for m in (a, b):
        m.couple(thermostat=True, barostat="isotropic", seed=12, n_steps=20)
        m.prime()
    assert a._paint_fused and not b._paint_fused
    for m in (a, b):
        m.capture()
        m.run(5)
    torch.cuda.synchronize()
    assert rel_rms(a.r.cpu().numpy(), b.r.cpu().numpy()) < 1e-6
    assert rel_rms(a.v.cpu().numpy(), b.v.cpu().numpy()) < 1e-5
    assert rel_rms(a.f_field.cpu().numpy(), b.f_field.cpu().numpy()) < 1e-5
    assert np.allclose(a.box_now(), b.box_now(), rtol=1e-7)
    assert not np.allclose(a.box_now(), np.asarray(cfg.box()), rtol=1e-9)  # the box moved
    a.check_errors()
    b.check_errors()


def test_fused_paint_refuses_semiisotropic_barostat():
    """The semi-isotropic position update leaves most beads unscaled while
    the box changes, so the paint is not fused (the MD loop keeps the
    separate paint) and the C entry point refuses the combination."""
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    s = systems.lipid_membrane(seed=9, n_lipids=60, n_water=900, box=5.6, mesh=24)
    cfg = s["config"]
    cfg.tau_p, cfg.n_b = 1.0, 1
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, get_hamiltonian(cfg),
                 topology=s["topology"])
    md.couple(thermostat=True, barostat="semiisotropic", seed=3, n_steps=5,
              target_pressure=(1.0, 1.0))
    assert not md._paint_fused
    md.prime()
    md.step()
    torch.cuda.synchronize()
    md.check_errors()


def test_charge_chain_with_no_charged_beads():
    """Charges given but all zero: the charge chain runs on an empty list of
    charged beads (no deposits, a zero field), and the step equals the one
    without charges."""
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    s = systems.charged_peptides(seed=14, n_chains=8, n_res=10, n_total=3000, box=6.0, mesh=24)
    cfg = s["config"]
    ham = get_hamiltonian(cfg)
    a = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"],
                charges=np.zeros(len(s["types"]), np.float32))
    b = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    assert a.charged.numel() == 0
    for m in (a, b):
        m.couple(thermostat=True, seed=2, n_steps=10)
        m.prime()
        m.capture()
        m.run(3)
    torch.cuda.synchronize()
    assert torch.count_nonzero(a.f_elec) == 0
    assert torch.equal(a.r, b.r) and torch.equal(a.v, b.v)
    a.check_errors()


def test_fused_paint_without_free_beads():
    """A melt where every bead is bonded: no free-bead kernel to fork, the
    deposits all come from the molecule groups; same trajectory as the
    separate paint."""
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    s = systems.homopolymer_melt(seed=15, n_chains=200, length=10, box=5.5, mesh=24)
    cfg = s["config"]
    ham = get_hamiltonian(cfg)
    a = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    b = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    b.FUSE_PAINT = False
    assert a._free_ids.numel() == 0 and a._paint_fused
    for m in (a, b):
        m.prime()
        m.capture()
        m.run(4)
    torch.cuda.synchronize()
    assert torch.equal(a.r, b.r) and torch.equal(a.v, b.v)
    assert torch.equal(a.f_field, b.f_field)
    a.check_errors()


def test_resort_with_fused_paint_and_barostat():
    """Re-sorting a captured NPT system whose paint is fused into the rRESPA
    launch: the trajectory in the caller's order follows the run without
    re-sorts to rounding (the barostat's sums run in another order)."""
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    s = systems.lipid_membrane(seed=10, n_lipids=60, n_water=900, box=5.6, mesh=24)
    cfg = s["config"]
    cfg.tau_p, cfg.n_b = 1.0, 1
    ham = get_hamiltonian(cfg)
    a = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    b = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"])
    for m in (a, b):
        m.couple(thermostat=True, barostat="isotropic", seed=6, n_steps=20)
        m.prime()
        m.capture()
    assert a._paint_fused
    a.resort_every = 2
    a.run(6)
    b.run(6)
    torch.cuda.synchronize()
    assert a.resorts == 3
    assert rel_rms(a.in_input_order(a.r).cpu().numpy(), b.r.cpu().numpy()) < 1e-6
    assert rel_rms(a.in_input_order(a.v).cpu().numpy(), b.v.cpu().numpy()) < 1e-4
    assert np.allclose(a.box_now(), b.box_now(), rtol=1e-6)
    a.check_errors()


@pytest.mark.parametrize("kind", ["membrane", "charged"])
def test_barostat_scaling_in_readout_matches_scaling_kernel(kind):
    """With the fused paint under the isotropic barostat the density readout
    scales the positions by alpha as it reads them (hpf_field_pic_step with
    painted and pos_scale); against hpf_scr_scale_positions followed by the
    field step on the scaled positions, the same float products in another
    launch, positions, velocities, forces and box are bit-identical over
    eager and captured NPT (CSVR + SCR) steps."""
    from hymd_gb300 import _lib, systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD

    class ScaleKernel(RespaMD):
        def _outer_rest(self, st, fused=True):
            if not (fused and self._paint_fused and self.baro_args is not None):
                return super()._outer_rest(st, fused)
            _lib.call("hpf_scr_scale_positions", _lib.ptr(self.r), self.n,
                      _lib.ptr(self.state), 0, st)
            thermo = self.thermo_args is not None
            self._field(st, self.field_sums, kick=self._kick_args(thermo), painted=True)
            if thermo:
                _lib.call("hpf_csvr_scale", _lib.ptr(self.v), _lib.ptr(self.group), self.n,
                          _lib.ptr(self.state), int(self.thermo_args.remove_com), st)

    if kind == "membrane":
        s = systems.lipid_membrane(seed=9, n_lipids=60, n_water=900, box=5.6, mesh=24)
        kw = dict(topology=s["topology"])
    else:
        s = systems.charged_peptides(seed=8, n_chains=10, n_res=25, n_total=5000, box=7.5,
                                     mesh=32)
        kw = dict(topology=s["topology"], charges=s["charges"])
    cfg = s["config"]
    cfg.tau_p, cfg.n_b = 1.0, 1
    ham = get_hamiltonian(cfg)
    a = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, **kw)
    b = ScaleKernel(s["positions"], s["velocities"], s["types"], cfg, ham, **kw)
    for m in (a, b):
        m.couple(thermostat=True, barostat="isotropic", seed=12, n_steps=20)
        m.prime()
        m.run(2)
    assert a._paint_fused and b._paint_fused
    for m in (a, b):
        m.capture()
        m.run(4)
    torch.cuda.synchronize()
    names = ["r", "v", "f_field", "box"] + (["f_elec"] if kind == "charged" else [])
    for name in names:
        assert torch.equal(getattr(a, name), getattr(b, name)), name
    assert not np.allclose(a.box_now(), np.asarray(cfg.box()), rtol=1e-9)  # the box moved
    a.check_errors()
    b.check_errors()
