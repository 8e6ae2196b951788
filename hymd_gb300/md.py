"""GPU-resident rRESPA driver (the loop of hymd/main.py:764-1169).

One outer step, as in the reference:
  1. outer half kick with the slow forces (field [+ PIC] [+ dipole]),
     dt_outer = respa_inner * time_step                     (main.py:802-827)
  2. respa_inner times: half kick with the bonded forces, drift, wrap
     np.mod(r, box), bonded forces, half kick              (main.py:830-887)
  3. slow forces at the new positions: field (paint -> r2c -> fused k-space
     -> c2r -> readout) and, with charges, PIC_Spectral     (main.py:975-1095)
  4. second outer half kick                                 (main.py:1143-1169)
The half kick closing inner step i and the one opening step i+1 run in one
launch (two FP32 roundings, as two reference calls).  The whole step is a
fixed launch sequence with no host synchronisation, so `capture()` records it
once in a CUDA graph and `run()` replays it.
"""
import numpy as np
import torch

from . import _lib
from .field import ParticleMesh
from .force import BondedTopology


class RespaMD:
    def __init__(self, positions, velocities, types, config, hamiltonian, topology=None,
                 charges=None, device="cuda"):
        self.device = torch.device(device)
        self.config = config
        self.r = torch.as_tensor(np.asarray(positions, np.float32), device=self.device).contiguous()
        self.v = torch.as_tensor(np.asarray(velocities, np.float32), device=self.device).contiguous()
        self.types = torch.as_tensor(np.asarray(types, np.int32), device=self.device).contiguous()
        self.n = self.r.shape[0]
        self.T = int(config.n_types)
        self.pm = ParticleMesh(config.mesh_size, config.box_size, self.T, device=self.device)
        self.pm.set_functional(hamiltonian)
        self.box = self.pm.box_tensor()
        self.masses = _lib.dvec(list(config.m) if config.m else [1.0] * self.T)
        self.mass = float(config.mass)
        self.dt = float(config.time_step)
        self.respa = int(config.respa_inner)
        z = lambda: torch.zeros((self.n, 3), dtype=torch.float32, device=self.device)
        self.f_field, self.f_bond, self.f_angle, self.f_dih = z(), z(), z(), z()
        self.topo = topology if (topology is None or isinstance(topology, BondedTopology)) \
            else BondedTopology(topology, device=self.device)
        self.charges = None
        self.f_elec = None
        if charges is not None:
            self.charges = torch.as_tensor(np.asarray(charges, np.float32), device=self.device)
            self.f_elec = z()
            self.elec_factor = config.coulomb_constant / config.dielectric_const
        self.ws_bond = _lib.new_workspace(self.device)
        self.ws_angle = _lib.new_workspace(self.device)
        self.ws_dih = _lib.new_workspace(self.device)
        self.err = torch.zeros(8, dtype=torch.int32, device=self.device)
        self.field_sums = torch.zeros(8, dtype=torch.float64, device=self.device)
        if self.topo is not None and self.topo.n_dihedrals:
            nd = self.topo.n_dihedrals
            self.dipoles = torch.zeros((nd, 4, 3), dtype=torch.float32, device=self.device)
            self.transfer = torch.zeros((nd, 6, 3, 3), dtype=torch.float32, device=self.device)
        self.graph = None
        # kernels of this library launched per outer step (cuFFT's own
        # kernels and memsets not counted): 2 outer kicks, per inner step one
        # kick/drift plus one per bonded term kind, one closing kick, and the
        # field step (paint, paint finalize, k-space, readout) [+ PIC: paint,
        # finalize, k-space, readout]
        t = self.topo
        kinds = 0 if t is None else (int(t.n_bonds > 0) + int(t.n_angles > 0)
                                     + int(t.n_dihedrals > 0))
        self.launches_per_step = (2 + self.respa * (1 + kinds) + 1 + 4
                                  + (4 if charges is not None else 0))

    # ------------------------------------------------------------------
    def _slow_forces(self):
        return [f for f in (self.f_field, self.f_elec) if f is not None]

    def _outer_kick(self, st):
        fs = self._slow_forces()
        arr = (_lib.P * len(fs))(*[_lib.ptr(f) for f in fs])
        _lib.call("hpf_kick", _lib.ptr(self.v), arr, len(fs), self.n, self.mass,
                  self.respa * self.dt, st)

    def _bonded(self, st, dipole_flag):
        t = self.topo
        if t is None:
            return
        err = _lib.ctypes.c_void_p(self.err.data_ptr())
        box = _lib.ptr(self.box)
        if t.n_bonds:
            _lib.call("hpf_bonds", _lib.ptr(self.f_bond), _lib.ptr(self.r), self.n, box,
                      _lib.ptr(t.bond_a), _lib.ptr(t.bond_b), _lib.ptr(t.bond_r0),
                      _lib.ptr(t.bond_k), t.n_bonds, _lib.ptr(self.ws_bond), err, st)
        if t.n_angles:
            _lib.call("hpf_angles", _lib.ptr(self.f_angle), _lib.ptr(self.r), self.n, box,
                      _lib.ptr(t.ang_a), _lib.ptr(t.ang_b), _lib.ptr(t.ang_c), _lib.ptr(t.ang_t0),
                      _lib.ptr(t.ang_k), t.n_angles, _lib.ptr(self.ws_angle), err, st)
        if t.n_dihedrals:
            _lib.call("hpf_dihedrals", _lib.ptr(self.f_dih), _lib.ptr(self.r), self.n,
                      _lib.ptr(self.dipoles), _lib.ptr(self.transfer), box, _lib.ptr(t.dih_a),
                      _lib.ptr(t.dih_b), _lib.ptr(t.dih_c), _lib.ptr(t.dih_d),
                      _lib.ptr(t.dih_coeff), _lib.ptr(t.dih_type), _lib.ptr(t.dih_last),
                      t.n_dihedrals, int(dipole_flag), _lib.ptr(self.ws_dih), err, st)

    def _bonded_ptrs(self):
        t = self.topo
        if t is None:
            return None, None, None
        return (_lib.ptr(self.f_bond) if t.n_bonds else None,
                _lib.ptr(self.f_angle) if t.n_angles else None,
                _lib.ptr(self.f_dih) if t.n_dihedrals else None)

    def _field(self, st, sums=None):
        _lib.call("hpf_field_step", self.pm._h, _lib.ptr(self.r), _lib.ptr(self.types), self.n,
                  self.masses, _lib.ptr(self.f_field), _lib.ptr(sums), st)
        if self.charges is not None:
            _lib.call("hpf_pic_step", self.pm._h, _lib.ptr(self.r), _lib.ptr(self.charges),
                      self.n, float(self.elec_factor), _lib.ptr(self.f_elec), None, None, None,
                      None, None, st)

    def prime(self):
        """Bonded and slow forces at the initial positions (main.py:494-588)."""
        st = _lib.stream_ptr()
        self._bonded(st, 0)
        self._field(st)

    def step(self):
        """One outer rRESPA step (launch sequence only; no host sync)."""
        st = _lib.stream_ptr()
        fb, fa, fd = self._bonded_ptrs()
        self._outer_kick(st)
        for inner in range(self.respa):
            kicks = 1 if inner == 0 else 2
            _lib.call("hpf_inner_kick_drift", _lib.ptr(self.r), _lib.ptr(self.v), fb, fa, fd,
                      self.n, self.mass, self.dt, kicks, 1, _lib.ptr(self.box), st)
            self._bonded(st, 1 if inner == self.respa - 1 else 0)
        _lib.call("hpf_inner_kick_drift", _lib.ptr(self.r), _lib.ptr(self.v), fb, fa, fd, self.n,
                  self.mass, self.dt, 1, 0, None, st)
        self._field(st)
        self._outer_kick(st)

    def capture(self):
        """Record one outer step in a CUDA graph (after a warm-up step)."""
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.step()
        torch.cuda.current_stream(self.device).wait_stream(s)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step()
        self.graph = g
        return g

    def run(self, steps):
        for _ in range(steps):
            if self.graph is not None:
                self.graph.replay()
            else:
                self.step()

    # ------------------------------------------------------------------
    def energies(self):
        """(bond, angle, dihedral) energies of the last inner step (FP64)."""
        out = []
        t = self.topo
        for ws, n in ((self.ws_bond, t.n_bonds if t else 0), (self.ws_angle, t.n_angles if t else 0),
                      (self.ws_dih, t.n_dihedrals if t else 0)):
            out.append(float(ws[0].item()) if n else 0.0)
        return out

    def check_errors(self):
        code = int(self.err[0].item())
        self.pm.check_errors()
        if code:
            raise _lib.HPFError("bonded device check", code)
