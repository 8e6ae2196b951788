"""Seeded synthetic systems of the benchmark workloads (no external data).

  homopolymer_melt   10k beads: 1000 chains x 10 (500 all-A, 500 all-B),
                     box 10 nm, mesh 32^3, chi_AB = 15, bonds r0 0.47 / k 1250
  lipid_membrane     162k beads: 6000 12-bead lipids (N,P,G,G, two C4 tails)
                     in two leaflets at z = +-2 nm + 90k W, box 27 nm,
                     mesh 64^3, chi_CW=30, chi_CN=chi_CP=15, chi_CG=6, chi_GW=4
  charged_peptides   500k beads: 200 chains x 50 (BB+SC) residues, 20% of
                     SC charged +-1 e with counter-ions, W solvent, box 40 nm,
                     mesh 128^3, dihedrals (cosine series + CBT), eps_r = 80
Velocities are Maxwell-Boltzmann at the stated temperature for mass 72.
Topologies are built with the host topology code (force.prepare_bonds) on
one molecule and tiled, which gives the same arrays as running it on the
whole system (the per-molecule lists are concatenated in molecule order).
Each builder also returns the whole system's bond rows (`bonds`, the
reference's (N, M) input form) for prepare_bonds on the full system.
"""
import numpy as np

from .config import Config
from .force import Angle, Bond, Chi, Dihedral, prepare_bonds

KB = 0.0083144621


def _velocities(rng, n, T, mass):
    return rng.normal(0.0, np.sqrt(KB * T / mass), size=(n, 3)).astype(np.float32)


def _random_walk(rng, start, n, step):
    d = rng.normal(size=(n - 1, 3))
    d *= step / np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([start[None, :], start[None, :] + np.cumsum(d, axis=0)])


def _tile_topology(template, n_mol, mol_size, n_total):
    """Concatenate the packed arrays of identical molecules placed at
    consecutive index blocks."""
    (b2a, b2b, b2r, b2k, b3a, b3b, b3c, b3t, b3k,
     b4a, b4b, b4c, b4d, coeff, b4t, last) = template
    off = (np.arange(n_mol) * mol_size)[:, None]
    tile_i = lambda x: (x[None, :] + off).reshape(-1)
    tile_f = lambda x: np.tile(x, n_mol)
    return (tile_i(b2a), tile_i(b2b), tile_f(b2r), tile_f(b2k),
            tile_i(b3a), tile_i(b3b), tile_i(b3c), tile_f(b3t), tile_f(b3k),
            tile_i(b4a), tile_i(b4b), tile_i(b4c), tile_i(b4d),
            np.tile(coeff, (n_mol, 1, 1)), tile_f(b4t), tile_f(last))


def _tile_rows(conn, n_mol, mol_size, n_total):
    """Bond rows of the whole system in the reference's input form (N, M):
    identical molecules at consecutive index blocks, -1 for no partner and
    for the beads after the molecules."""
    conn = np.asarray(conn)
    rows = np.full((n_total, conn.shape[1]), -1, dtype=np.int64)
    off = (np.arange(n_mol) * mol_size)[:, None, None]
    rows[:n_mol * mol_size] = np.where(conn[None] >= 0, conn[None] + off, -1).reshape(-1,
                                                                                    conn.shape[1])
    return rows


def _config(**kw):
    c = Config(n_steps=kw.pop("n_steps", 1000), time_step=kw.pop("time_step", 0.03),
               mesh_size=kw.pop("mesh_size"), sigma=kw.pop("sigma", 0.5),
               kappa=kw.pop("kappa", 0.05))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def homopolymer_melt(seed=1, n_chains=1000, length=10, box=10.0, mesh=32, chi_ab=15.0):
    rng = np.random.default_rng(seed)
    L = np.full(3, box)
    N = n_chains * length
    r = np.concatenate([_random_walk(rng, rng.uniform(0, box, 3), length, 0.47)
                        for _ in range(n_chains)])
    r = np.mod(r, L).astype(np.float32)
    types = np.repeat(np.arange(n_chains) >= n_chains // 2, length).astype(np.int32)
    names = np.where(types == 0, b"A", b"B")
    molecules = np.repeat(np.arange(n_chains), length)
    idx = np.arange(length)
    conn = np.full((length, 3), -1)
    conn[1:, 0] = idx[:-1]
    conn[:-1, 1] = idx[1:]
    cfg = _config(mesh_size=mesh, box_size=L, n_particles=N, n_types=2, mass=72.0,
                  respa_inner=10, time_step=0.03, target_temperature=323.0, tau=0.1,
                  hamiltonian="DefaultWithChi", unique_names=["A", "B"],
                  type_to_name_map={0: "A", 1: "B"}, m=[1.0, 1.0],
                  chi=[Chi("A", "B", float(chi_ab))],
                  bonds=[Bond("A", "A", 0.47, 1250.0), Bond("B", "B", 0.47, 1250.0)])
    # A and B chains have the same bond parameters, so one template serves both
    tmpl = prepare_bonds(np.zeros(length, int), np.full(length, b"A"), conn, idx, cfg)
    topo = _tile_topology(tmpl, n_chains, length, N)
    v = _velocities(rng, N, 323.0, 72.0)
    return dict(positions=r, velocities=v, types=types, names=names, molecules=molecules,
                topology=topo, config=cfg, bonds=_tile_rows(conn, n_chains, length, N))


# dppc-like lipid: N(0)-P(1)-G(2)-C(4)-C(5)-C(6)-C(7); G(2)-G(3)-C(8)-C(9)-C(10)-C(11)
_LIPID_NAMES = [b"N", b"P", b"G", b"G", b"C", b"C", b"C", b"C", b"C", b"C", b"C", b"C"]
_LIPID_CONN = np.array([[1, -1, -1], [0, 2, -1], [1, 3, 4], [2, 8, -1], [2, 5, -1], [4, 6, -1],
                        [5, 7, -1], [6, -1, -1], [3, 9, -1], [8, 10, -1], [9, 11, -1],
                        [10, -1, -1]])
# depth (in bond lengths from the head) and lateral tail offset of each bead
_LIPID_DEPTH = np.array([0, 1, 2, 2, 3, 4, 5, 6, 3, 4, 5, 6], dtype=np.float64)
_LIPID_SIDE = np.array([0, 0, -1, 1, -1, -1, -1, -1, 1, 1, 1, 1], dtype=np.float64)


def lipid_membrane(seed=2, n_lipids=6000, n_water=90000, box=27.0, mesh=64, chi_cw=30.0):
    rng = np.random.default_rng(seed)
    L = np.full(3, box)
    zc = box / 2
    per = n_lipids // 2
    g = int(np.ceil(np.sqrt(per)))
    xs = (np.arange(g) + 0.5) * box / g
    grid = np.stack(np.meshgrid(xs, xs, indexing="ij"), -1).reshape(-1, 2)
    lip = []
    for leaflet, sgn in ((0, 1.0), (1, -1.0)):
        sel = rng.permutation(len(grid))[:per if leaflet == 0 else n_lipids - per]
        for (x, y) in grid[sel]:
            pos = np.zeros((12, 3))
            pos[:, 0] = x + 0.25 * _LIPID_SIDE
            pos[:, 1] = y
            pos[:, 2] = zc + sgn * (2.0 - 0.47 * _LIPID_DEPTH * 0.55)
            pos += rng.normal(0.0, 0.1, size=(12, 3))
            lip.append(pos)
    lip = np.concatenate(lip)
    # solvent uniformly in the volume outside the bilayer slab |z - zc| <= 2.6
    w = np.empty((0, 3))
    while len(w) < n_water:
        c = rng.uniform(0, box, size=(n_water, 3))
        w = np.concatenate([w, c[np.abs(c[:, 2] - zc) > 2.6]])
    w = w[:n_water]
    r = np.mod(np.concatenate([lip, w]), L).astype(np.float32)
    uniq = ["C", "G", "N", "P", "W"]
    tmap = {u.encode(): i for i, u in enumerate(uniq)}
    names = np.array(_LIPID_NAMES * n_lipids + [b"W"] * n_water)
    types = np.array([tmap[x] for x in names], dtype=np.int32)
    N = len(r)
    molecules = np.concatenate([np.repeat(np.arange(n_lipids), 12),
                                n_lipids + np.arange(n_water)])
    chi = [Chi("C", "W", float(chi_cw)), Chi("C", "N", 15.0), Chi("C", "P", 15.0), Chi("C", "G", 6.0),
           Chi("G", "W", 4.0)]
    bonds = [Bond(a, b, 0.47, 1250.0) for a, b in
             (("N", "P"), ("P", "G"), ("G", "G"), ("G", "C"), ("C", "C"))]
    angles = [Angle(atom_1=a, atom_2=b, atom_3=c, equilibrium=eq, strength=25.0)
              for a, b, c, eq in (("P", "G", "G", 120.0), ("P", "G", "C", 180.0),
                                  ("G", "C", "C", 180.0), ("C", "C", "C", 180.0))]
    cfg = _config(mesh_size=mesh, box_size=L, n_particles=N, n_types=5, mass=72.0,
                  respa_inner=10, time_step=0.03, target_temperature=323.0, tau=0.1,
                  hamiltonian="DefaultWithChi", unique_names=uniq,
                  type_to_name_map=dict(enumerate(uniq)), m=[1.0] * 5, chi=chi, bonds=bonds,
                  angle_bonds=angles, barostat="isotropic", tau_p=1.0, n_b=1)
    tmpl = prepare_bonds(np.zeros(12, int), np.array(_LIPID_NAMES), _LIPID_CONN,
                         np.arange(12), cfg)
    topo = _tile_topology(tmpl, n_lipids, 12, N)
    v = _velocities(rng, N, 323.0, 72.0)
    cfg.rho0 = N / float(np.prod(L))
    cfg.a = cfg.rho0
    return dict(positions=r, velocities=v, types=types, names=names, molecules=molecules,
                topology=topo, config=cfg, bonds=_tile_rows(_LIPID_CONN, n_lipids, 12, N))


def charged_peptides(seed=3, n_chains=200, n_res=50, n_total=500_000, box=40.0, mesh=128):
    rng = np.random.default_rng(seed)
    L = np.full(3, box)
    per = 2 * n_res
    chains = []
    for _ in range(n_chains):
        bb = _random_walk(rng, rng.uniform(0, box, 3), n_res, 0.38)
        d = rng.normal(size=(n_res, 3))
        d *= 0.3 / np.linalg.norm(d, axis=1, keepdims=True)
        res = np.empty((per, 3))
        res[0::2] = bb
        res[1::2] = bb + d
        chains.append(res)
    pep = np.concatenate(chains)
    n_pep = len(pep)
    sc_idx = np.arange(n_pep)[1::2]
    charged = rng.permutation(sc_idx)[: int(0.2 * len(sc_idx))]
    q = np.zeros(n_total, np.float32)
    q[charged] = rng.choice([-1.0, 1.0], size=len(charged))
    net = int(round(q.sum()))
    n_ions = abs(net)
    n_w = n_total - n_pep
    w = rng.uniform(0, box, size=(n_w, 3))
    r = np.mod(np.concatenate([pep, w]), L).astype(np.float32)
    q[n_pep:n_pep + n_ions] = -np.sign(net) if net else 0.0
    uniq = ["BB", "SC", "W"]
    names = np.array(([b"BB", b"SC"] * n_res) * n_chains + [b"W"] * n_w)
    types = np.array([0, 1] * n_res * n_chains + [2] * n_w, dtype=np.int32)
    molecules = np.concatenate([np.repeat(np.arange(n_chains), per),
                                n_chains + np.arange(n_w)])
    chi_v = rng.uniform(0, 25, 3)
    chi = [Chi("BB", "SC", chi_v[0]), Chi("BB", "W", chi_v[1]), Chi("SC", "W", chi_v[2])]
    cfg = _config(mesh_size=mesh, box_size=L, n_particles=n_total, n_types=3, mass=72.0,
                  respa_inner=10, time_step=0.03, target_temperature=323.0, tau=0.1,
                  hamiltonian="DefaultWithChi", unique_names=uniq,
                  type_to_name_map=dict(enumerate(uniq)), m=[1.0] * 3, chi=chi,
                  coulombtype="PIC_Spectral", dielectric_const=80.0,
                  type_charges=[0.0, 0.0, 0.0])
    # one chain's topology: BB-BB and BB-SC bonds, BB-BB-BB angles, BB4 dihedrals
    conn = np.full((per, 3), -1)
    for i in range(n_res):
        b = 2 * i
        nb = [b + 1]
        if i > 0:
            nb.append(b - 2)
        if i < n_res - 1:
            nb.append(b + 2)
        conn[b, :len(nb)] = nb
        conn[b + 1, 0] = b
    coeffs = np.zeros((6, 5))
    coeffs[0, :4] = rng.normal(0, 2, 4)
    coeffs[1, :4] = rng.uniform(-np.pi, np.pi, 4)
    coeffs[4, :3] = np.abs(rng.normal(0, 20, 3))
    coeffs[5, :3] = rng.uniform(-np.pi, np.pi, 3)
    cfg.bonds = [Bond("BB", "BB", 0.38, 1250.0), Bond("BB", "SC", 0.30, 1250.0)]
    cfg.angle_bonds = [Angle(atom_1="BB", atom_2="BB", atom_3="BB", equilibrium=120.0,
                             strength=25.0)]
    cfg.dihedrals = [Dihedral("BB", "BB", "BB", "BB", coeffs, 1)]
    tmpl = prepare_bonds(np.zeros(per, int), np.array([b"BB", b"SC"] * n_res), conn,
                         np.arange(per), cfg)
    topo = _tile_topology(tmpl, n_chains, per, n_total)
    v = _velocities(rng, n_total, 323.0, 72.0)
    cfg.rho0 = n_total / float(np.prod(L))
    cfg.a = cfg.rho0
    return dict(positions=r, velocities=v, types=types, names=names, molecules=molecules,
                topology=topo, config=cfg, charges=q,
                bonds=_tile_rows(conn, n_chains, per, n_total))


BUILDERS = {"melt10k": homopolymer_melt, "membrane162k": lipid_membrane,
            "peptide500k": charged_peptides}

REPLICA_MESHES = (32, 48, 64, 96)


def replica_set(n_replicas=64, seed=5, n_min=5_000, n_max=200_000, density=8.3, spacing=0.4):
    """Independent replicas mixing the melt and membrane recipes: bead counts
    log-uniform in [n_min, n_max], cubic box for `density` beads/nm^3, mesh
    from REPLICA_MESHES closest to box/spacing, chi_AB (melt) or chi_CW
    (membrane) uniform in [5, 40] kJ/mol.  Even indices are melts, odd ones
    membranes (44% of the beads in 12-bead lipids, as in the 162k membrane)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_replicas):
        n = float(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        chi = float(rng.uniform(5.0, 40.0))
        sub = int(rng.integers(1 << 30))
        if i % 2 == 0:
            n_chains = max(2, int(round(n / 10)))
            N = 10 * n_chains
        else:
            n_lipids = max(2, int(round(0.44 * n / 12)))
            n_water = max(1, int(round(n)) - 12 * n_lipids)
            N = 12 * n_lipids + n_water
        box = (N / density) ** (1.0 / 3.0)
        mesh = min(REPLICA_MESHES, key=lambda m: abs(m - box / spacing))
        if i % 2 == 0:
            s = homopolymer_melt(seed=sub, n_chains=n_chains, box=box, mesh=mesh, chi_ab=chi)
        else:
            s = lipid_membrane(seed=sub, n_lipids=n_lipids, n_water=n_water, box=box, mesh=mesh,
                               chi_cw=chi)
        s["recipe"] = "melt" if i % 2 == 0 else "membrane"
        s["chi"] = chi
        out.append(s)
    return out
