"""Bonded interactions on GB300 -- drop-in for hymd/force.py.

Topology preparation (host, bit-exact with the reference):
  prepare_bonds_old          hymd/force.py:325-505
  prepare_index_based_bonds  hymd/force.py:508-570
  prepare_bonds              hymd/force.py:573-728
  propensity_potential_coeffs hymd/force.py:280-322
The reference builds a networkx graph per molecule and walks it with
all_pairs_shortest_path and a recursive path enumeration; the order of the
resulting term lists is fixed by those traversals.  This module performs the
same traversals (breadth-first search with neighbours in insertion order,
depth-first enumeration of simple 4-paths) on plain adjacency dictionaries,
over molecules grouped once instead of rescanning all particles per molecule,
so the lists come out identical, in the same order.

Force kernels (device, libhpf_gb300.so), in the f2py calling form used by
hymd/main.py:509-550:
  compute_bond_forces(f, r, box, a, b, r0, k) -> (energy, bond_pr)
  compute_angle_forces(f, r, box, a, b, c, t0, k) -> (energy, angle_pr)
  compute_dihedral_forces(f, r, dipoles, transfer, box, a, b, c, d, coeff,
                          dtype, last, dipole_flag) -> energy
  dipole_forces_redistribution(f_on_bead, f_dipoles, trans_matrices, a, b, c,
                               d, type_array, last_bb)
f, dipoles, transfer are CUDA tensors written in place; index/parameter
arrays may be numpy (copied per call) or prepared device tensors
(`BondedTopology`).
"""
import logging
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib

log = logging.getLogger(__name__)


@dataclass
class Dielectric_type:
    atom_1: str
    dielectric_value: float


@dataclass
class Bond:
    atom_1: str
    atom_2: str
    equilibrium: float
    strength: float


@dataclass
class Angle(Bond):
    atom_3: str


@dataclass
class Dihedral:
    atom_1: str
    atom_2: str
    atom_3: str
    atom_4: str
    coeffs: np.ndarray
    dih_type: int


@dataclass
class Chi:
    atom_1: str
    atom_2: str
    interaction_energy: float


# ---------------------------------------------------------------- topology ---
_ALPHA = ([7.406, -5.298, -2.570, 1.336, 0.739],
          [-0.28632126, 1.2099146, 1.18122138, 0.49075168, 0.98495911])
_BETA = ([3.770, 5.929, -4.151, -0.846, 0.190],
         [-0.2300693, -0.0583289, 0.99342396, 1.03237971, 2.90160988])
_COIL = ([1.416, -0.739, 0.990, -0.397, 0.136],
         [1.3495933, 0.45649087, 2.30441057, -0.12274901, -0.26179939])


def propensity_potential_coeffs(x: float):
    """Cosine-series coefficients for coiling propensity lambda = x in [-1, 1]
    (hymd/force.py:280-322; Bore et al., JCTC 14, 1120 (2018)).

    Returns a (4, 5) array: rows 0-1 the alpha (x<0) or beta (x>0) series
    scaled by (|x| -+ x)/2, rows 2-3 the coil series scaled by 1 - |x|; at
    x = -1, 0, 1 the pure alpha / coil / beta series and two zero rows.
    """
    alpha = np.array(_ALPHA)
    beta = np.array(_BETA)
    coil = np.array(_COIL)
    zero = np.zeros((2, 5))
    if np.isclose(x, -1):
        return np.concatenate((alpha, zero))
    if np.isclose(x, 0):
        return np.concatenate((coil, zero))
    if np.isclose(x, 1):
        return np.concatenate((beta, zero))
    ax = abs(x)
    if ax > 1:
        log.error("The provided value of lambda = %s is out of lambda definition range, "
                  "[-1.0, 1.0].", x)
        return None
    coil[0] *= 1 - ax
    if x < 0:
        alpha[0] *= 0.5 * (ax - x)
        return np.concatenate((alpha, coil))
    beta[0] *= 0.5 * (ax + x)
    return np.concatenate((beta, coil))


def _name(x):
    return x.decode("UTF-8") if isinstance(x, (bytes, np.bytes_)) else str(x)


def _molecule_groups(molecules):
    """Unique molecule ids (ascending) with their member local indices in
    ascending order."""
    molecules = np.asarray(molecules)
    order = np.argsort(molecules, kind="stable")
    ids, starts = np.unique(molecules[order], return_index=True)
    ends = np.append(starts[1:], len(order))
    return [(ids[i], order[starts[i]:ends[i]]) for i in range(len(ids))]


def _bfs_paths(adj, src):
    """Shortest paths from src in breadth-first discovery order, neighbours
    visited in insertion order (the order networkx's
    single_source_shortest_path produces)."""
    paths = {src: [src]}
    level = [src]
    while level:
        nxt = []
        for v in level:
            for w in adj[v]:
                if w not in paths:
                    paths[w] = paths[v] + [w]
                    nxt.append(w)
        level = nxt
    return paths


def _simple_paths(adj, u, n):
    """All simple paths with n further nodes starting at u, depth first,
    neighbours in insertion order."""
    if n == 0:
        return [[u]]
    out = []
    for w in adj[u]:
        for p in _simple_paths(adj, w, n - 1):
            if u not in p:
                out.append([u] + p)
    return out


def _dihedral_classes(dihedral_types):
    """Class of each dihedral type: the index of the first type with equal
    coefficients and dihedral type.  The reference's duplicate test
    (force.py:476-487, `... not in bonds_4`) compares a reversed term by its indices, coefficients
    and type, so types equal in both are one type for it."""
    cls = []
    for i, a in enumerate(dihedral_types):
        c = i
        for j in range(i):
            b = dihedral_types[j]
            if (a.dih_type == b.dih_type and np.shape(a.coeffs) == np.shape(b.coeffs)
                    and np.array_equal(np.asarray(a.coeffs), np.asarray(b.coeffs))):
                c = cls[j]
                break
        cls.append(c)
    return cls


def prepare_bonds_old(molecules, names, bonds, indices, config):
    """hymd/force.py:325-505 -> (bonds_2, bonds_3, bonds_4, bb_index)."""
    bonds_2, bonds_3, bonds_4, bb_index = [], [], [], []
    seen4 = set()
    dihedral_types = list(config.dihedrals)
    dcls = _dihedral_classes(dihedral_types)
    for _, members in _molecule_groups(molecules):
        bb_dihedral = 0
        adj = {}
        attr = {}
        for li in members:
            gi = indices[li]
            gi = gi.item() if hasattr(gi, "item") else gi
            adj.setdefault(gi, {})
            attr[gi] = (_name(names[li]), int(li))
            for bnd in bonds[li]:
                if bnd == -1:
                    continue
                bnd = bnd.item() if hasattr(bnd, "item") else bnd
                adj.setdefault(bnd, {})
                adj[gi].setdefault(bnd, None)
                adj[bnd].setdefault(gi, None)
        adj = {k: list(v) for k, v in adj.items()}
        for i in list(adj):
            for j, path in _bfs_paths(adj, i).items():
                if len(path) == 2 and path[-1] > path[0]:
                    ni, nj = attr[i][0], attr[j][0]
                    for b in config.bonds:
                        if (ni == b.atom_1 and nj == b.atom_2) or (ni == b.atom_2 and nj == b.atom_1):
                            bonds_2.append([attr[i][1], attr[j][1], b.equilibrium, b.strength])
                if len(path) == 3 and path[-1] > path[0]:
                    ni, nm, nj = attr[i][0], attr[path[1]][0], attr[j][0]
                    for a in config.angle_bonds:
                        fwd = ni == a.atom_1 and nm == a.atom_2 and nj == a.atom_3
                        bwd = ni == a.atom_3 and nm == a.atom_2 and nj == a.atom_1
                        if fwd or bwd:
                            bonds_3.append([attr[i][1], attr[path[1]][1], attr[j][1],
                                            np.radians(a.equilibrium), a.strength])
            for p in _simple_paths(adj, i, 3):
                nm = [attr[x][0] for x in p]
                loc = [attr[x][1] for x in p]
                for ti, a in enumerate(dihedral_types):
                    if (nm[0] == a.atom_1 and nm[1] == a.atom_2 and nm[2] == a.atom_3
                            and nm[3] == a.atom_4):
                        if (loc[3], loc[2], loc[1], loc[0], dcls[ti]) in seen4:
                            continue
                        bonds_4.append([loc[0], loc[1], loc[2], loc[3], a.coeffs, a.dih_type])
                        seen4.add((loc[0], loc[1], loc[2], loc[3], dcls[ti]))
                        if a.dih_type == 1:
                            bb_dihedral = len(bonds_4)
        if bb_dihedral:
            bb_index.append(bb_dihedral - 1)
    return bonds_2, bonds_3, bonds_4, bb_index


def prepare_index_based_bonds(molecules, topol):
    """hymd/force.py:508-570 (topology given per residue name)."""
    bonds_2, bonds_3, bonds_4 = [], [], []
    summary = topol["system"]["molecules"]
    for mol, members in _molecule_groups(molecules):
        resid = mol + 1
        resname = None
        total = 0
        for entry in summary:
            total += entry[1]
            if resid <= total:
                resname = entry[0]
                break
        if resname is None:
            break
        first = int(members[0])
        block = topol[resname]
        for bond in block.get("bonds", []):
            bonds_2.append([bond[0] - 1 + first, bond[1] - 1 + first, bond[3], bond[4]])
        for ang in block.get("angles", []):
            bonds_3.append([ang[0] - 1 + first, ang[1] - 1 + first, ang[2] - 1 + first,
                            np.radians(ang[4]), ang[5]])
        for dih in block.get("dihedrals", []):
            dih_type = dih[4]
            coeff = dih[5]
            if dih_type == 0 and isinstance(coeff[0], (float, int)):
                coeff = propensity_potential_coeffs(coeff[0])
            elif dih_type == 1 and len(coeff) == 3:
                coeff = np.array(propensity_potential_coeffs(coeff[0][0]).tolist() + coeff[1:])
            elif dih_type == 2:
                coeff = np.array(coeff)
            else:
                coeff = np.insert(np.array(coeff), 2, np.zeros((2, 5)), axis=0)
            bonds_4.append([dih[0] - 1 + first, dih[1] - 1 + first, dih[2] - 1 + first,
                            dih[3] - 1 + first, coeff, dih_type, 0])
    return bonds_2, bonds_3, bonds_4


def _topology_device(molecules, names, bonds, indices, config, device):
    """prepare_bonds_old's term discovery on the device (hpf_topology_terms):
    the host maps names, term types and global indices to small integers
    (numpy, vectorised); one device thread per molecule walks the molecule's
    graph in the reference's traversal order.  Returns the packed arrays of
    prepare_bonds (numpy, same dtypes)."""
    dev = torch.device(device)
    molecules = np.asarray(molecules)
    N = len(molecules)
    order = np.argsort(molecules, kind="stable")
    _, starts = np.unique(molecules[order], return_index=True)
    mol_start = np.append(starts, N).astype(np.int32)
    n_mol = len(starts)
    bead_slot = np.empty(N, np.int32)
    bead_slot[order] = np.arange(N, dtype=np.int32)
    uniq, name_id = np.unique(np.asarray(names), return_inverse=True)
    nid = {_name(u): i for i, u in enumerate(uniq)}
    gidx = np.asarray(indices).astype(np.int64).reshape(N)
    rows = np.asarray(bonds).astype(np.int64).reshape(N, -1)
    sorter = np.argsort(gidx, kind="stable")
    sg = gidx[sorter]
    valid = rows != -1
    pos = np.minimum(np.searchsorted(sg, rows), max(N - 1, 0))
    found = (sg[pos] == rows) if N else valid
    if np.any(valid & ~found):
        raise ValueError("prepare_bonds: a bond names a particle index that is not present")
    partners = np.where(valid, sorter[pos], -1).astype(np.int32)
    name = lambda x: nid.get(x, -1)
    bt = np.array([[name(b.atom_1), name(b.atom_2)] for b in config.bonds], np.int32)
    at = np.array([[name(a.atom_1), name(a.atom_2), name(a.atom_3)] for a in config.angle_bonds],
                  np.int32)
    dts = list(config.dihedrals)
    dt = np.array([[name(a.atom_1), name(a.atom_2), name(a.atom_3), name(a.atom_4)] for a in dts],
                  np.int32)
    dcls = np.array(_dihedral_classes(dts), np.int32)
    dbb = np.array([int(a.dih_type == 1) for a in dts], np.int32)
    i32 = lambda x: torch.as_tensor(np.ascontiguousarray(x, dtype=np.int32).reshape(-1),
                                    device=dev)
    d_ms, d_sb, d_bs = i32(mol_start), i32(order), i32(bead_slot)
    d_gid = torch.as_tensor(gidx, device=dev)
    d_nid, d_par = i32(name_id), i32(partners)
    d_bt, d_at, d_dt, d_cls, d_bb = i32(bt), i32(at), i32(dt), i32(dcls), i32(dbb)
    scratch = torch.empty(max(int(_lib.lib().hpf_topology_scratch_ints(N)), 1), dtype=torch.int32,
                          device=dev)
    counts = torch.zeros((max(n_mol, 1), 3), dtype=torch.int32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    st = _lib.stream_ptr()
    common = (N, n_mol, _lib.ptr(d_ms), _lib.ptr(d_sb), _lib.ptr(d_bs), _lib.ptr(d_gid),
              _lib.ptr(d_nid), _lib.ptr(d_par), rows.shape[1], _lib.ptr(d_bt), len(bt),
              _lib.ptr(d_at), len(at), _lib.ptr(d_dt), _lib.ptr(d_cls), _lib.ptr(d_bb), len(dts),
              _lib.ptr(scratch))
    _lib.call("hpf_topology_terms", *common, _lib.ptr(counts), None, None, None, None, None,
              _lib.ptr(err), st)
    csum = torch.cumsum(counts.to(torch.int64), dim=0)
    offsets = (csum - counts).to(torch.int32).contiguous()
    B, A, D = (int(x) for x in csum[-1].tolist())
    e = int(err.item())
    if e:
        raise _lib.HPFError("hpf_topology_terms", e)
    t2 = torch.empty((max(B, 1), 3), dtype=torch.int32, device=dev)
    t3 = torch.empty((max(A, 1), 4), dtype=torch.int32, device=dev)
    t4 = torch.empty((max(D, 1), 5), dtype=torch.int32, device=dev)
    bbm = torch.empty(max(n_mol, 1), dtype=torch.int32, device=dev)
    _lib.call("hpf_topology_terms", *common, _lib.ptr(counts), _lib.ptr(offsets), _lib.ptr(t2),
              _lib.ptr(t3), _lib.ptr(t4), _lib.ptr(bbm), _lib.ptr(err), st)
    t2, t3, t4 = t2[:B].cpu().numpy(), t3[:A].cpu().numpy(), t4[:D].cpu().numpy()
    bbm = bbm[:n_mol].cpu().numpy()
    e = int(err.item())
    if e:
        raise _lib.HPFError("hpf_topology_terms", e)
    r0 = np.array([b.equilibrium for b in config.bonds], np.float64)
    kb = np.array([b.strength for b in config.bonds], np.float64)
    t0 = np.array([np.radians(a.equilibrium) for a in config.angle_bonds], np.float64)
    ka = np.array([a.strength for a in config.angle_bonds], np.float64)
    ctab = np.array([np.resize(a.coeffs, (6, 5)) for a in dts], np.float64).reshape(-1, 6, 5)
    ttab = np.array([a.dih_type for a in dts], int)
    ix = lambda c: c.astype(int)
    last = np.zeros(D, dtype=int)
    last[bbm[bbm >= 0]] = 1
    return (ix(t2[:, 0]), ix(t2[:, 1]), r0[t2[:, 2]], kb[t2[:, 2]],
            ix(t3[:, 0]), ix(t3[:, 1]), ix(t3[:, 2]), t0[t3[:, 3]], ka[t3[:, 3]],
            ix(t4[:, 0]), ix(t4[:, 1]), ix(t4[:, 2]), ix(t4[:, 3]),
            ctab[t4[:, 4]] if D else np.empty((0, 6, 5)), ttab[t4[:, 4]], last)


def prepare_bonds(molecules, names, bonds, indices, config, topol=None, device=None):
    """hymd/force.py:573-728: the 16 packed arrays for the bonded kernels.

    Dihedral coefficients are np.resize'd to (6, 5) (a 2- or 4-row set is
    repeated cyclically, as in the reference).  With `device` (e.g. "cuda")
    and no `topol`, the term discovery of prepare_bonds_old runs on that
    device (one thread per molecule) and gives the same arrays."""
    if topol is None and device is not None:
        return _topology_device(molecules, names, bonds, indices, config, device)
    if topol is not None:
        b2, b3, b4 = prepare_index_based_bonds(molecules, topol)
        bb_index = None
    else:
        b2, b3, b4, bb_index = prepare_bonds_old(molecules, names, bonds, indices, config)
    B, A, D = len(b2), len(b3), len(b4)
    b2a = np.array([x[0] for x in b2], dtype=int).reshape(B)
    b2b = np.array([x[1] for x in b2], dtype=int).reshape(B)
    b2r = np.array([x[2] for x in b2], dtype=np.float64).reshape(B)
    b2k = np.array([x[3] for x in b2], dtype=np.float64).reshape(B)
    b3a = np.array([x[0] for x in b3], dtype=int).reshape(A)
    b3b = np.array([x[1] for x in b3], dtype=int).reshape(A)
    b3c = np.array([x[2] for x in b3], dtype=int).reshape(A)
    b3t = np.array([x[3] for x in b3], dtype=np.float64).reshape(A)
    b3k = np.array([x[4] for x in b3], dtype=np.float64).reshape(A)
    b4 = list(b4)
    b4a = np.array([x[0] for x in b4], dtype=int).reshape(D)
    b4b = np.array([x[1] for x in b4], dtype=int).reshape(D)
    b4c = np.array([x[2] for x in b4], dtype=int).reshape(D)
    b4d = np.array([x[3] for x in b4], dtype=int).reshape(D)
    coeff = np.empty((D, 6, 5), dtype=np.float64)
    b4t = np.empty(D, dtype=int)
    last = np.zeros(D, dtype=int)
    for i, x in enumerate(b4):
        coeff[i] = np.resize(x[4], (6, 5))
        b4t[i] = x[5]
        if topol is not None:
            last[i] = x[6]
    if topol is None:
        last[bb_index] = 1
    return (b2a, b2b, b2r, b2k, b3a, b3b, b3c, b3t, b3k, b4a, b4b, b4c, b4d, coeff, b4t, last)


# ------------------------------------------------------------ device side ---
class BondedTopology:
    """Device copies of the packed bonded arrays (int32 indices, float32
    parameters, float32 (D,6,5) coefficients -- the Fortran reads coeff as
    real(4) in both precisions)."""

    def __init__(self, packed, device="cuda"):
        (b2a, b2b, b2r, b2k, b3a, b3b, b3c, b3t, b3k,
         b4a, b4b, b4c, b4d, coeff, b4t, last) = packed
        i32 = lambda x: torch.as_tensor(np.asarray(x, dtype=np.int32), device=device)
        f32 = lambda x: torch.as_tensor(np.asarray(x, dtype=np.float32), device=device)
        self.bond_a, self.bond_b, self.bond_r0, self.bond_k = i32(b2a), i32(b2b), f32(b2r), f32(b2k)
        self.ang_a, self.ang_b, self.ang_c = i32(b3a), i32(b3b), i32(b3c)
        self.ang_t0, self.ang_k = f32(b3t), f32(b3k)
        self.dih_a, self.dih_b, self.dih_c, self.dih_d = i32(b4a), i32(b4b), i32(b4c), i32(b4d)
        self.dih_coeff = f32(np.asarray(coeff).reshape(-1, 6, 5))
        self.dih_type, self.dih_last = i32(b4t), i32(last)
        self.n_bonds, self.n_angles, self.n_dihedrals = len(b2a), len(b3a), len(b4a)
        self.has_cbt = bool(np.any(np.asarray(b4t) == 1))


_WS = {}


def _ws(device, key):
    k = (str(device), key)
    if k not in _WS:
        _WS[k] = _lib.new_workspace(device)
    return _WS[k]


def _dev_i32(x, device):
    if isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == torch.int32:
        return x.contiguous()
    return torch.as_tensor(np.asarray(x if not isinstance(x, torch.Tensor) else x.cpu(),
                                      dtype=np.int32), device=device)


def _dev_f32(x, device):
    if isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == torch.float32:
        return x.contiguous()
    return torch.as_tensor(np.asarray(x if not isinstance(x, torch.Tensor) else x.cpu(),
                                      dtype=np.float32), device=device)


def _dev_box(box, device):
    if isinstance(box, torch.Tensor) and box.is_cuda and box.dtype == torch.float64:
        return box
    return torch.as_tensor(np.asarray(box, dtype=np.float64).reshape(3), device=device)


def _err(device):
    """Device int32 error word shared by the bonded entry points."""
    k = (str(device), "err")
    if k not in _WS:
        _WS[k] = torch.zeros(8, dtype=torch.int32, device=device)
    return _WS[k]


def _check_err(device):
    e = _err(device)
    code = int(e[0].item())
    if code:
        e.zero_()
        raise _lib.HPFError("bonded device check", int(code))


# Every device argument below is bound to a local name until the library call
# has been issued: a temporary that died earlier would return its memory to
# torch's caching allocator, and the next temporary could reuse it before the
# kernel reads it.

def compute_bond_forces(f, r, box, a, b, r0, k, sync=True):
    """cbf (hymd/compute_bond_forces.f90:1-61) -> (energy, bond_pr).

    With sync=False returns the device workspace whose [0:4] hold
    (energy, bond_pr) and does not synchronise."""
    _lib.require_cuda(f, "f", torch.float32)
    _lib.require_cuda(r, "r", torch.float32)
    dev = r.device
    ws, err = _ws(dev, "bonds"), _err(dev)
    bx = _dev_box(box, dev)
    A, B = _dev_i32(a, dev), _dev_i32(b, dev)
    R0, K = _dev_f32(r0, dev), _dev_f32(k, dev)
    _lib.call("hpf_bonds", _lib.ptr(f), _lib.ptr(r), r.shape[0], _lib.ptr(bx), _lib.ptr(A),
              _lib.ptr(B), _lib.ptr(R0), _lib.ptr(K), A.numel(), _lib.ptr(ws), _lib.ptr(err),
              _lib.stream_ptr())
    if not sync:
        return ws
    out = ws[:4].cpu().numpy()
    _check_err(dev)
    return float(out[0]), out[1:4].astype(np.float32)


def compute_angle_forces(f, r, box, a, b, c, t0, k, sync=True):
    """caf (hymd/compute_angle_forces.f90:1-93) -> (energy, angle_pr)."""
    _lib.require_cuda(f, "f", torch.float32)
    _lib.require_cuda(r, "r", torch.float32)
    dev = r.device
    ws, err = _ws(dev, "angles"), _err(dev)
    bx = _dev_box(box, dev)
    A, B, C = _dev_i32(a, dev), _dev_i32(b, dev), _dev_i32(c, dev)
    T0, K = _dev_f32(t0, dev), _dev_f32(k, dev)
    _lib.call("hpf_angles", _lib.ptr(f), _lib.ptr(r), r.shape[0], _lib.ptr(bx), _lib.ptr(A),
              _lib.ptr(B), _lib.ptr(C), _lib.ptr(T0), _lib.ptr(K), A.numel(), _lib.ptr(ws),
              _lib.ptr(err), _lib.stream_ptr())
    if not sync:
        return ws
    out = ws[:4].cpu().numpy()
    _check_err(dev)
    return float(out[0]), out[1:4].astype(np.float32)


def compute_dihedral_forces(f, r, dipoles, transfer, box, a, b, c, d, coeff, dtype, last,
                            dipole_flag, sync=True):
    """cdf (hymd/compute_dihedral_forces.f90:1-137) -> energy.  dipoles
    (D,4,3) and transfer (D,6,3,3) are zeroed and, with dipole_flag=1,
    filled for CBT (type 1) terms."""
    _lib.require_cuda(f, "f", torch.float32)
    _lib.require_cuda(r, "r", torch.float32)
    dev = r.device
    ws, err = _ws(dev, "dihedrals"), _err(dev)
    bx = _dev_box(box, dev)
    A, B, C, Dd = (_dev_i32(x, dev) for x in (a, b, c, d))
    nd = A.numel()
    cf = _dev_f32(coeff, dev).reshape(nd, 6, 5).contiguous()
    ty, la = _dev_i32(dtype, dev), _dev_i32(last, dev)
    _lib.require_cuda(dipoles, "dipoles", torch.float32, (nd, 4, 3))
    _lib.require_cuda(transfer, "transfer", torch.float32, (nd, 6, 3, 3))
    _lib.call("hpf_dihedrals", _lib.ptr(f), _lib.ptr(r), r.shape[0], _lib.ptr(dipoles),
              _lib.ptr(transfer), _lib.ptr(bx), _lib.ptr(A), _lib.ptr(B), _lib.ptr(C),
              _lib.ptr(Dd), _lib.ptr(cf), _lib.ptr(ty), _lib.ptr(la), nd, int(dipole_flag),
              _lib.ptr(ws), _lib.ptr(err), _lib.stream_ptr())
    if not sync:
        return ws
    e = float(ws[0].item())
    _check_err(dev)
    return e


def dipole_forces_redistribution(f_on_bead, f_dipoles, trans_matrices, a, b, c, d, type_array,
                                 last_bb):
    """hymd/force.py:855-877: zero f_on_bead and add the transfer-matrix
    images of the dipole pseudo-charge forces (CBT dihedrals only)."""
    _lib.require_cuda(f_on_bead, "f_on_bead", torch.float32)
    dev = f_on_bead.device
    A, B, C, Dd = (_dev_i32(x, dev) for x in (a, b, c, d))
    nd = A.numel()
    fd = _dev_f32(f_dipoles, dev).reshape(nd, 4, 3).contiguous()
    tm = _dev_f32(trans_matrices, dev).reshape(nd, 6, 3, 3).contiguous()
    ty, la = _dev_i32(type_array, dev), _dev_i32(last_bb, dev)
    _lib.call("hpf_dipole_redistribute", _lib.ptr(f_on_bead), f_on_bead.shape[0], _lib.ptr(fd),
              _lib.ptr(tm), _lib.ptr(A), _lib.ptr(B), _lib.ptr(C), _lib.ptr(Dd), _lib.ptr(ty),
              _lib.ptr(la), nd, _lib.stream_ptr())
