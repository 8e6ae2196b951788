"""GPU-resident rRESPA driver (the loop of hymd/main.py:764-1169).

One outer step, as in the reference:
  1. outer half kick with the slow forces (field [+ PIC]),
     dt_outer = respa_inner * time_step                     (main.py:802-827)
  2. respa_inner times: half kick with the bonded forces, drift, wrap
     np.mod(r, box), bonded forces, half kick              (main.py:830-887)
  3. slow forces at the new positions: field (paint -> r2c -> fused k-space
     -> c2r -> readout) and, with charges, PIC_Spectral     (main.py:975-1095)
  4. second outer half kick                                 (main.py:1143-1169)

fused=True (default): steps 1-2 are one launch of the molecule-blocked
rRESPA kernel (hpf_respa_step); molecules that do not fit a CTA fall back to
the per-term kernels.  fused=False: per-term kernels and one kick/drift
launch per inner step (the reference's call sequence, kept for comparison).
Either way a step is a fixed launch sequence with no host synchronisation, so
`capture()` records it once in a CUDA graph and `run()` replays it.
"""
import numpy as np
import torch

from . import _lib
from .field import ParticleMesh
from .force import BondedTopology


class RespaMD:
    def __init__(self, positions, velocities, types, config, hamiltonian, topology=None,
                 charges=None, device="cuda", fused=True, max_block_beads="auto"):
        self.device = torch.device(device)
        self.config = config
        self.r = torch.as_tensor(np.asarray(positions, np.float32), device=self.device).contiguous()
        self.v = torch.as_tensor(np.asarray(velocities, np.float32), device=self.device).contiguous()
        self.types = torch.as_tensor(np.asarray(types, np.int32), device=self.device).contiguous()
        self.n = self.r.shape[0]
        self.T = int(config.n_types)
        self.pm = ParticleMesh(config.mesh_size, config.box_size, self.T, device=self.device)
        self.pm.set_functional(hamiltonian)
        self._hamiltonian = hamiltonian
        self.box = self.pm.box_tensor()
        self.masses = _lib.dvec(list(config.m) if config.m else [1.0] * self.T)
        self.mass = float(config.mass)
        self.dt = float(config.time_step)
        self.respa = int(config.respa_inner)
        z = lambda: torch.zeros((self.n, 3), dtype=torch.float32, device=self.device)
        self.f_field, self.f_bond, self.f_angle, self.f_dih = z(), z(), z(), z()
        self.f_b = z()  # combined bonded force carried by the fused kernel
        packed = None
        if topology is None or isinstance(topology, BondedTopology):
            self.topo = topology
        else:
            packed = topology
            self.topo = BondedTopology(topology, device=self.device)
        self.charges = None
        self.f_elec = None
        self.charged = None
        if charges is not None:
            self.charges = torch.as_tensor(np.asarray(charges, np.float32), device=self.device)
            self.f_elec = z()
            self._index_charged()
            self.elec_factor = config.coulomb_constant / config.dielectric_const
        self.ws_bond = _lib.new_workspace(self.device)
        self.ws_angle = _lib.new_workspace(self.device)
        self.ws_dih = _lib.new_workspace(self.device)
        self.bonded_out = torch.zeros(16, dtype=torch.float64, device=self.device)
        self.err = torch.zeros(8, dtype=torch.int32, device=self.device)
        self.dipoles = self.transfer = None
        if self.topo is not None and self.topo.n_dihedrals:
            nd = self.topo.n_dihedrals
            self.dipoles = torch.zeros((nd, 4, 3), dtype=torch.float32, device=self.device)
            self.transfer = torch.zeros((nd, 6, 3, 3), dtype=torch.float32, device=self.device)
        self.plan = None
        self.block_timings = None
        self.spectral_tile_timings = None
        self._packed = packed
        self.block_beads = None
        self.perm = None  # memory order -> input order, after sort_particles()
        # bead order of the mesh-cell sort: "molecule" keeps each molecule's
        # beads together (ordered by the cell of one bead of the molecule),
        # "bead" sorts every bead by its own cell
        self.sort_order = "molecule"
        self._mol = None  # per bead: a bead of its molecule (int32, device)
        self._free_ids = None  # the plan's free beads, ascending (int32, device)
        self._inv_acc = None  # composed re-sorts not yet applied to the host topology
        self._packed_dirty = False
        self._resort_graph = None
        self.resort_every = 0  # run(): re-sort by mesh cell every this many steps
        self.resorts = 0
        self.steps_run = 0
        if fused and self.topo is not None and packed is not None:
            if max_block_beads == "auto":
                self.plan = self._tune_plan(packed)
            else:
                self.plan = self._make_plan(packed, max_block_beads)
                self.block_beads = int(max_block_beads)
            self._index_free()
        self.graph = None
        self.graph_inner = self.graph_field = None
        self.field_sums = torch.zeros(8, dtype=torch.float64, device=self.device)
        self.thermo_args = None
        self.baro_args = None
        self.baro_mode = 0
        self.counter = torch.zeros(4, dtype=torch.int32, device=self.device)
        self.state = torch.zeros(16, dtype=torch.float64, device=self.device)
        self.ws_md = _lib.new_workspace(self.device)
        self.names = None
        # PLUMED-style bias (set_bias): a host callback every outer step
        self.bias = None
        self.f_bias = None
        self.bias_indices = None
        self.plumed_bias = 0.0
        self.step_count = 0
        t = self.topo
        kinds = 0 if t is None else (int(t.n_bonds > 0) + int(t.n_angles > 0)
                                     + int(t.n_dihedrals > 0))
        # kernels of this library per outer step (cuFFT's own kernels and
        # memsets not counted): a field evaluation is paint, spectral passes
        # A, B, C and readout on the fused path, paint, finalize, k-space and
        # readout around cuFFT otherwise; PIC adds a second one
        per_field = 5 if self.pm.spectral == "fused" else 4
        field = per_field * (2 if charges is not None else 1)
        if self.plan is not None:
            # fused inner kernel + its one-block finish (sums, barostat); the
            # second kick is fused into the readout
            self._launches = 2 + field
        else:
            self._launches = 1 + self.respa * (1 + kinds) + 1 + field

    def _make_plan(self, packed, max_block_beads):
        (b2a, b2b, b2r, b2k, b3a, b3b, b3c, b3t, b3k,
         b4a, b4b, b4c, b4d, coeff, b4t, last) = packed
        i32 = lambda x: np.ascontiguousarray(np.asarray(x, dtype=np.int32))
        f32 = lambda x: np.ascontiguousarray(np.asarray(x, dtype=np.float32))
        arrs = [i32(b2a), i32(b2b), f32(b2r), f32(b2k), i32(b3a), i32(b3b), i32(b3c), f32(b3t),
                f32(b3k), i32(b4a), i32(b4b), i32(b4c), i32(b4d),
                f32(np.asarray(coeff).reshape(-1, 6, 5)), i32(b4t), i32(last)]
        p = lambda a: a.ctypes.data_as(_lib.P)
        h = _lib.P()
        code = _lib.lib().hpf_respa_plan_create(
            _lib.ctypes.byref(h), self.n, len(arrs[0]), *[p(a) for a in arrs[0:4]],
            len(arrs[4]), *[p(a) for a in arrs[4:9]], len(arrs[9]), *[p(a) for a in arrs[9:16]],
            int(max_block_beads))
        if code == 7:  # a molecule larger than a CTA can hold
            return None
        if code:
            raise _lib.HPFError("hpf_respa_plan_create", code)
        return h

    # group sizes tried by the autotuner (beads per molecule group)
    BLOCK_CANDIDATES = (12, 16, 24, 32, 36, 48, 64)

    def _tune_plan(self, packed, reps=4):
        """Molecule-group size of the fused inner kernel picked by timing it on
        this system: each candidate plan runs `reps` launches (CUDA events) on
        a copy of the state; the fastest is kept.  Candidates that give the
        same grouping are timed once.  Timings (us) are kept in
        `block_timings`."""
        r, v = self.r.clone(), self.v.clone()
        fb, slow = torch.zeros_like(self.r), torch.zeros_like(self.r)
        arr = (_lib.P * 1)(_lib.ptr(slow))
        st = _lib.stream_ptr()
        best, seen, timings = None, set(), {}
        for c in self.BLOCK_CANDIDATES:
            plan = self._make_plan(packed, c)
            if plan is None:
                continue
            a, b, m = _lib.I(), _lib.I(), _lib.I()
            _lib.call("hpf_respa_plan_info", plan, _lib.ctypes.byref(a), _lib.ctypes.byref(b),
                      _lib.ctypes.byref(m))
            key = (a.value, m.value)
            if key in seen:
                _lib.lib().hpf_respa_plan_destroy(plan)
                continue
            seen.add(key)

            def launch():
                _lib.call("hpf_respa_step", plan, _lib.ptr(r), _lib.ptr(v), _lib.ptr(fb), arr, 1,
                          self.mass, self.dt, self.respa, _lib.ptr(self.box), None, None, None,
                          None, None, None, None, None, None, _lib.ptr(self.err), st)

            launch()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                launch()
            e1.record()
            e1.synchronize()
            t = e0.elapsed_time(e1) * 1000.0 / reps
            timings[c] = t
            if best is None or t < best[0]:
                if best is not None:
                    _lib.lib().hpf_respa_plan_destroy(best[1])
                best = (t, plan, c)
            else:
                _lib.lib().hpf_respa_plan_destroy(plan)
        self.err.zero_()
        self.block_timings = timings
        if best is None:
            return None
        self.block_beads = best[2]
        return best[1]

    # per-bead arrays that sort_particles() permutes together
    _PER_BEAD = ("r", "v", "types", "charges", "f_field", "f_elec", "f_bias", "f_b", "f_bond",
                 "f_angle",
                 "f_dih", "group")

    def sort_particles(self, order=None):
        """Reorder the beads in memory by mesh cell (x-major cell index,
        stable), so that neighbouring threads of the paint and readout touch
        neighbouring mesh points.  order="molecule" (the default,
        `sort_order`) keeps the beads of a molecule together, ordered by the
        cell of one bead of the molecule, so that the bonded kernels still
        read each molecule from one stretch of memory; order="bead" sorts each
        bead by its own cell.  Every per-bead array is permuted in place and
        the bonded topology and the fused plan are rebuilt with the new
        indices; the physics is unchanged.  `perm` maps memory order to the
        caller's order (`in_input_order`).  Call before capture() (a captured
        graph holds the old plan); resort() re-sorts a captured system."""
        if self.graph is not None or self.graph_inner is not None:
            raise RuntimeError("sort_particles() must come before capture()")
        if order is not None:
            if order not in ("molecule", "bead"):
                raise ValueError(f"unknown sort order {order!r}")
            self.sort_order = order
        self._sync_packed()
        self._index_molecules()
        perm = self._cell_order()
        inv = torch.empty_like(perm)
        inv[perm] = torch.arange(self.n, device=self.device)
        for name in self._PER_BEAD:
            t = getattr(self, name, None)
            if t is not None:
                t.copy_(t[perm])
        if self._mol is not None:
            self._mol.copy_(inv[self._mol[perm].long()].to(torch.int32))
        if self._packed is not None:
            inv_h = inv.cpu().numpy()
            packed = list(self._packed)
            for k in self._PACKED_IDS:
                packed[k] = inv_h[np.asarray(packed[k], dtype=np.int64)].astype(np.int32)
            self._packed = tuple(packed)
            self.topo = BondedTopology(self._packed, device=self.device)
            if self.plan is not None:
                _lib.lib().hpf_respa_plan_destroy(self.plan)
                self.plan = self._make_plan(self._packed, self.block_beads)
                self._index_free()
        self.perm = perm if self.perm is None else self.perm[perm]
        if self.charges is not None:
            self._index_charged()
        return self.perm

    # bead index arrays of the packed topology (bonds a, b; angles a, b, c;
    # dihedrals a, b, c, d)
    _PACKED_IDS = (0, 1, 4, 5, 6, 9, 10, 11, 12)

    def _bonded_pairs(self):
        """Both ends of every bond and of the consecutive bead pairs of every
        angle and dihedral (device int64), or None without a topology."""
        t = self.topo
        if t is None:
            return None
        pairs = [(t.bond_a, t.bond_b), (t.ang_a, t.ang_b), (t.ang_b, t.ang_c),
                 (t.dih_a, t.dih_b), (t.dih_b, t.dih_c), (t.dih_c, t.dih_d)]
        pairs = [(a, b) for a, b in pairs if a.numel()]
        if not pairs:
            return None
        return (torch.cat([a.long() for a, _ in pairs]), torch.cat([b.long() for _, b in pairs]))

    def _index_molecules(self):
        """Per bead, the smallest bead index of its molecule (the connected
        component of the bonded terms), by label propagation with pointer
        jumping; a free bead is its own molecule.  Kept (and permuted) for the
        "molecule" sort order."""
        if self.sort_order != "molecule" or self._mol is not None:
            return
        lab = torch.arange(self.n, device=self.device)
        pairs = self._bonded_pairs()
        if pairs is not None:
            a, b = pairs
            while True:
                m = torch.minimum(lab[a], lab[b])
                new = lab.clone()
                new.scatter_reduce_(0, a, m, "amin")
                new.scatter_reduce_(0, b, m, "amin")
                new = new[new]
                if torch.equal(new, lab):
                    break
                lab = new
        self._mol = lab.to(torch.int32)

    def _index_free(self):
        """The plan's free beads (in no bonded term) in ascending order, kept
        beside the plan so that a re-sort hands it the new list in memory
        order."""
        if self.plan is None:
            self._free_ids = None
            return
        mask = torch.zeros(self.n, dtype=torch.bool, device=self.device)
        pairs = self._bonded_pairs()
        if pairs is not None:
            mask[pairs[0]] = True
            mask[pairs[1]] = True
        self._free_ids = torch.nonzero(~mask).reshape(-1).to(torch.int32).contiguous()
        nb, nf = _lib.I64(), _lib.I64()
        _lib.call("hpf_respa_plan_counts", self.plan, _lib.ctypes.byref(nb),
                  _lib.ctypes.byref(nf))
        if nf.value != self._free_ids.numel():
            raise RuntimeError("free-bead count differs from the plan's")

    def _cell_order(self):
        """Stable permutation of the beads by the x-major index of the mesh
        cell of their current position; in the "molecule" order by the cell
        of the molecule's first bead, then by that bead, so that each
        molecule stays in one stretch.  Capturable (no host copies)."""
        n1, n2 = self.pm.Nmesh[1], self.pm.Nmesh[2]
        if getattr(self, "_nmesh", None) is None:
            self._nmesh = torch.tensor(list(self.pm.Nmesh), dtype=torch.float64,
                                       device=self.device)
        nn = self._nmesh
        c = torch.floor(self.r.double() / self.box * nn).long()
        c = torch.remainder(c, nn.long())
        key = (c[:, 0] * n1 + c[:, 1]) * n2 + c[:, 2]
        if self.sort_order == "molecule" and self._mol is not None:
            mol = self._mol.long()
            key = key[mol] * self.n + mol
        return torch.argsort(key, stable=True)

    def resort(self):
        """Re-sort the beads by mesh cell between steps (the order the paint
        and readout want decays as beads move: at ~0.2 nm/ps a bead leaves
        its 0.3 nm cell within a few outer steps).  Unlike sort_particles()
        nothing is reallocated or rebuilt: every per-bead buffer is permuted
        in place, the fused plan's bead lists are remapped on the device
        (hpf_respa_plan_permute) with its free beads handed over again in
        ascending order, the bonded index arrays are remapped and the charged
        beads re-listed in ascending order, so graphs captured before stay
        valid.  Once the step is captured the re-sort is captured too (its
        own graph, replayed on later calls).  Per-bead results are
        unchanged; sums over beads (energies, CSVR) change in their last bits
        with the summation order.  `perm` follows."""
        if self.perm is None:
            self.perm = torch.arange(self.n, device=self.device)
        if self._inv_acc is None:
            self._inv_acc = torch.arange(self.n, device=self.device)
        if self.sort_order == "molecule" and self._mol is None:
            self._index_molecules()
        captured = self.graph is not None or self.graph_inner is not None
        if self._resort_graph is not None:
            self._resort_graph.replay()
        elif captured:
            # the first re-sort of a captured system runs on a side stream and
            # records the graph that later ones replay
            s = torch.cuda.Stream(device=self.device)
            s.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(s):
                self._resort_body()
            torch.cuda.current_stream(self.device).wait_stream(s)
            torch.cuda.synchronize(self.device)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self._resort_body()
            self._resort_graph = g
        else:
            self._resort_body()
        self._packed_dirty = True
        self.resorts += 1

    def _resort_body(self):
        """The device work of one re-sort; static shapes, no host copies."""
        p = self._cell_order()
        inv = torch.empty_like(p)
        inv.scatter_(0, p, torch.arange(self.n, device=self.device))
        inv32 = inv.to(torch.int32)
        for name in self._PER_BEAD:
            t = getattr(self, name, None)
            if t is not None:
                t.copy_(t[p])
        if self._mol is not None:
            self._mol.copy_(inv32[self._mol[p].long()])
        st = _lib.stream_ptr()
        if self.plan is not None:
            free = None
            if self._free_ids is not None and self._free_ids.numel():
                self._free_ids.copy_(torch.sort(inv32[self._free_ids.long()]).values)
                free = self._free_ids
            _lib.call("hpf_respa_plan_permute", self.plan, _lib.ptr(inv32), self.n,
                      None if free is None else _lib.ptr(free),
                      0 if free is None else free.numel(), _lib.ptr(self.err), st)
        t = self.topo
        if t is not None:
            for name in ("bond_a", "bond_b", "ang_a", "ang_b", "ang_c", "dih_a", "dih_b",
                         "dih_c", "dih_d"):
                a = getattr(t, name)
                if a.numel():
                    a.copy_(inv32[a.long()])
        if self.charged is not None and self.charged.numel():
            self.charged.copy_(torch.sort(inv32[self.charged.long()]).values)
        self.perm.copy_(self.perm[p])
        # the host copy of the topology follows when a plan is rebuilt
        self._inv_acc.copy_(inv[self._inv_acc])

    def _sync_packed(self):
        """Apply the re-sorts since the last plan build to the host topology."""
        if self._packed is None or not self._packed_dirty:
            return
        inv = self._inv_acc.cpu().numpy()
        packed = list(self._packed)
        for k in self._PACKED_IDS:
            packed[k] = inv[np.asarray(packed[k], dtype=np.int64)].astype(np.int32)
        self._packed = tuple(packed)
        self._inv_acc.copy_(torch.arange(self.n, device=self.device))
        self._packed_dirty = False

    def in_input_order(self, t):
        """A per-bead tensor (in memory order) returned in the caller's order."""
        if self.perm is None:
            return t
        out = torch.empty_like(t)
        out[self.perm] = t
        return out

    def couple(self, thermostat=True, barostat=None, seed=0, n_steps=100000, groups=None,
               remove_com=True, target_pressure=1.0, beta=7.6e-4):
        """Enable the CSVR thermostat (hymd/thermostat.py:111-219) and/or the
        SCR barostat on the device: barostat="isotropic"
        (hymd/barostat_scr.py:34-132, target_pressure in bar) or
        "semiisotropic" (:133-284, target_pressure = (P_L, P_N) in bar; a
        direction with a zero target is not coupled, as in the reference).

        The random numbers of `n_steps` outer steps are drawn now with
        numpy's default_rng(seed), in the reference's order per step: the
        barostat's normal() (semi-isotropic: lateral, then normal), then for
        each thermostat group normal() and chisquare(3 N_g - 1).  groups:
        optional int array (0/1) of coupling groups (default: one group of all
        particles)."""
        cfg = self.config
        every = int(cfg.n_b or 1)
        ng = 1
        self.group = None
        counts = [float(self.n), 0.0]
        if groups is not None:
            g = np.asarray(groups, np.int32)
            if self.perm is not None:  # groups come in the caller's order
                g = g[self.perm.cpu().numpy()]
            ng = int(g.max()) + 1
            if ng > 2:
                raise NotImplementedError("at most two thermostat coupling groups")
            self.group = torch.as_tensor(g, device=self.device)
            counts = [float(np.sum(g == 0)), float(np.sum(g == 1))]
        if barostat not in (None, False, "isotropic", "semiisotropic"):
            raise NotImplementedError(f"device barostat {barostat!r}")
        nbar = 2 if barostat == "semiisotropic" else 1
        stride = nbar + 2 * ng
        rng = np.random.default_rng(seed)
        table = np.zeros((n_steps, stride))
        for s in range(n_steps):
            if (s + 1) % every:
                continue
            if barostat:
                for q in range(nbar):
                    table[s, q] = rng.normal()
            if thermostat:
                for gi in range(ng):
                    table[s, nbar + 2 * gi] = rng.normal()
                    table[s, nbar + 1 + 2 * gi] = rng.chisquare(3 * int(counts[gi]) - 1)
        self.randoms = torch.as_tensor(table.reshape(-1), device=self.device)
        dt_o = self.respa * self.dt
        if thermostat:
            a = _lib.CsvrArgs()
            a.n_groups, a.remove_com, a.n_steps, a.stride = ng, int(remove_com), n_steps, stride
            a.offset, a.advance, a.every = nbar, 1, every
            a.count[0], a.count[1] = counts
            a.mass, a.gas_constant = self.mass, cfg.gas_constant
            a.target_temperature = float(cfg.target_temperature)
            a.c = float(np.exp(-dt_o / cfg.tau))
            self.thermo_args = a
        self.baro_mode = 0
        if barostat:
            b = _lib.ScrArgs()
            if barostat == "semiisotropic":
                p_l, p_n = target_pressure
                b.mode, b.couple_l, b.couple_n = 1, int(bool(p_l)), int(bool(p_n))
                b.target_pressure_n = float(p_n or 0.0)
                target_pressure = float(p_l or 0.0)
                self.baro_mode = 1
            b.n_types, b.n_steps, b.stride = self.T, n_steps, stride
            b.advance = 0 if thermostat else 1
            b.every = every
            types = self.types.cpu().numpy()
            m = np.asarray(list(cfg.m) if cfg.m else [1.0] * self.T, dtype=np.float64)
            mc = m * np.bincount(types, minlength=self.T)[: self.T]
            Q = np.asarray(self.pm._functional_Q, dtype=np.float64)
            b.half_mQm = float(0.5 * mc @ Q @ mc)
            b.mass, b.gas_constant = self.mass, cfg.gas_constant
            b.target_temperature = float(cfg.target_temperature)
            b.target_pressure = float(target_pressure)
            b.beta, b.tau_p, b.dt_outer, b.n_b = beta, float(cfg.tau_p), dt_o, float(every)
            self.baro_args = b
        if self.plan is not None:
            # CSVR: sums (with the fused second kick) + scale; the barostat runs
            # in the rRESPA finish kernel and the paint (semi-isotropic: a
            # position kernel of its own)
            self._launches += (1 if thermostat else 0) + self.baro_mode
        else:
            self._launches += (1 if thermostat else 0) + (2 if barostat else 0)
        # (the CSVR sums ride in the readout; its scaling is one more launch)

    def _thermostat(self, st, kick=False):
        """CSVR; with kick=True the second outer half kick runs in the same
        pass, just before the kinetic energy is taken."""
        fs = self._slow_forces() if kick else []
        arr = (_lib.P * max(1, len(fs)))(*[_lib.ptr(f) for f in fs])
        _lib.call("hpf_csvr", _lib.ptr(self.v), _lib.ptr(self.group), self.n, arr, len(fs),
                  self.respa * self.dt, _lib.ctypes.byref(self.thermo_args),
                  _lib.ptr(self.randoms), _lib.ptr(self.counter), _lib.ptr(self.state),
                  _lib.ptr(self.ws_md), _lib.ptr(self.err), st)

    def _barostat(self, st):
        _lib.call("hpf_scr_isotropic", self.pm._h, _lib.ptr(self.r), _lib.ptr(self.v), self.n,
                  _lib.ptr(self.field_sums), _lib.ptr(self.bonded_out),
                  _lib.ctypes.byref(self.baro_args), _lib.ptr(self.randoms),
                  _lib.ptr(self.counter), _lib.ptr(self.state), _lib.ptr(self.ws_md),
                  _lib.ptr(self.err), st)

    def box_now(self):
        return self.box.cpu().numpy().copy()

    def plan_info(self):
        if self.plan is None:
            return None
        a, b, c = _lib.I(), _lib.I(), _lib.I()
        _lib.call("hpf_respa_plan_info", self.plan, _lib.ctypes.byref(a), _lib.ctypes.byref(b),
                  _lib.ctypes.byref(c))
        return dict(mol_blocks=a.value, free_beads=b.value, max_block_beads=c.value)

    def __del__(self):
        if getattr(self, "plan", None) is not None:
            try:
                _lib.lib().hpf_respa_plan_destroy(self.plan)
            except Exception:
                pass
            self.plan = None

    # ------------------------------------------------------------------
    def _slow_forces(self):
        return [f for f in (self.f_field, self.f_elec, self.f_bias) if f is not None]

    # ---- PLUMED-style bias ----------------------------------------------------
    def set_bias(self, bias, indices=None):
        """Couple a bias with PlumedBias's prepare/calc interface
        (hymd_gb300.plumed, hymd/plumed.py:11-235).  After every field
        evaluation the positions and the current forces (field + bonded +
        electrostatic, main.py:1097-1141) go to the host in the caller's bead
        order with `indices` (global indices, default 0..N-1); the returned
        bias force joins the slow forces of the outer half kicks
        (main.py:808-812, 1150-1154).  The bias runs on the host between
        kernel launches, so a run with a bias is not captured in a graph."""
        if self.graph is not None or self.graph_inner is not None:
            raise RuntimeError("set_bias() must come before capture()")
        self.bias = bias
        self.bias_indices = (np.arange(self.n, dtype=np.intc) if indices is None
                             else np.asarray(indices, dtype=np.intc))
        self.f_bias = torch.zeros((self.n, 3), dtype=torch.float32, device=self.device)

    def potential_energy(self):
        """Bonded energies of the last inner step plus the FP64 field (and
        PIC electrostatic) energy of the current positions (host sync)."""
        from .field import energy_fp64
        cfg = self.config
        fac = (cfg.coulomb_constant / cfg.dielectric_const) if self.charges is not None else 0.0
        e = energy_fp64(self.pm, self.r, self.types, list(cfg.m) if cfg.m else [1.0] * self.T,
                        self._hamiltonian, charges=self.charges, elec_factor=fac)
        w = e["W"]
        if self.charges is not None:
            w += 0.5 * e["V"] * e["Eq"] - float(cfg.self_energy or 0.0)
        return w + sum(self.energies())

    def _bias_forces(self):
        """One bias evaluation at the current positions (synchronises)."""
        f = self.f_field + self.f_b
        if self.f_elec is not None:
            f = f + self.f_elec
        forces = self.in_input_order(f).cpu().numpy()
        pos = self.in_input_order(self.r).cpu().numpy()
        cfg = self.config
        cfg.box_size = self.box_now()
        q = (self.in_input_order(self.charges).cpu().numpy() if self.charges is not None
             else np.zeros(self.n))
        needs = self.bias.prepare(self.step_count, forces, pos, self.bias_indices, cfg, q)
        pot = self.potential_energy() if needs else 0.0
        fb, e = self.bias.calc(forces, pot)
        fb = torch.as_tensor(np.asarray(fb, np.float32), device=self.device)
        self.f_bias.copy_(fb if self.perm is None else fb[self.perm])
        self.plumed_bias = e

    def _outer_kick(self, st):
        fs = self._slow_forces()
        arr = (_lib.P * len(fs))(*[_lib.ptr(f) for f in fs])
        _lib.call("hpf_kick", _lib.ptr(self.v), arr, len(fs), self.n, self.mass,
                  self.respa * self.dt, st)

    def _bonded(self, st, dipole_flag):
        t = self.topo
        if t is None:
            return
        err = _lib.ptr(self.err)
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

    def _index_charged(self):
        """Indices of the charged beads (int32, device), the only ones the
        MD loop's charge paint visits."""
        self.charged = torch.nonzero(self.charges != 0).reshape(-1).to(torch.int32).contiguous()

    def _kick_args(self, thermostat):
        """HpfKick for the second outer half kick fused into the last readout
        (with the CSVR sums when the thermostat is on)."""
        k = _lib.Kick()
        k.v = self.v.data_ptr()
        if self.charges is not None:
            k.prev[0] = self.f_field.data_ptr()  # field first, then the electrostatic force
            k.n_prev = 1
        k.mass = self.mass
        k.dt_outer = self.respa * self.dt
        if thermostat:
            k.thermo = _lib.ctypes.pointer(self.thermo_args)
            k.group = self.group.data_ptr() if self.group is not None else None
            k.randoms = self.randoms.data_ptr()
            k.counter = self.counter.data_ptr()
            k.state = self.state.data_ptr()
            k.ws = self.ws_md.data_ptr()
            k.d_err = self.err.data_ptr()
        self._kick_keep = k
        return _lib.ctypes.byref(k)

    # charged systems: the density and charge chains of the field step run
    # on two streams (hpf_field_pic_step) rather than one after the other
    CONCURRENT_PIC = True
    # the fused rRESPA kernel deposits every bead on the mesh where it leaves
    # its final position (hpf_respa_step_paint), and the field step skips its
    # paints; with the isotropic barostat the deposits of the unscaled
    # positions in the old box are those of the scaled ones in the new box
    # (up to rounding), and the density readout scales the positions as it
    # reads them; not with the semi-isotropic one, whose position update leaves most
    # beads unscaled while the box changes
    FUSE_PAINT = True

    @property
    def launches_per_step(self):
        """Kernels of this library per outer step (cuFFT's own kernels and
        memsets not counted).  With the paint fused into the rRESPA kernel the
        field step's paints (densities, charges) are gone and the free beads
        run as a kernel of their own beside the groups."""
        n = self._launches
        if self._paint_fused:
            n -= 1 + (1 if self.charges is not None else 0)
            if self._free_ids is not None and self._free_ids.numel():
                n += 1
        return n

    @property
    def _paint_fused(self):
        return (self.FUSE_PAINT and self.plan is not None and self.pm.spectral == "fused"
                and (self.baro_args is None or self.baro_mode == 0)
                and (self.charges is None or self.CONCURRENT_PIC))

    def _field(self, st, sums=None, pos_scale=None, kick=None, painted=False):
        scale = None if pos_scale is None else _lib.ctypes.c_void_p(pos_scale)
        if (self.charges is not None and self.CONCURRENT_PIC) or painted:
            charged = self.charges is not None
            _lib.call("hpf_field_pic_step", self.pm._h, _lib.ptr(self.r), _lib.ptr(self.types),
                      self.n, self.masses, _lib.ptr(self.f_field), _lib.ptr(sums), scale,
                      _lib.ptr(self.charges) if charged else None,
                      _lib.ptr(self.charged) if charged else None,
                      self.charged.numel() if charged else 0,
                      float(self.elec_factor) if charged else 0.0,
                      _lib.ptr(self.f_elec) if charged else None, None, kick, int(painted), st)
            return
        last_kick = kick if self.charges is None else None
        _lib.call("hpf_field_step", self.pm._h, _lib.ptr(self.r), _lib.ptr(self.types), self.n,
                  self.masses, _lib.ptr(self.f_field), _lib.ptr(sums), scale, last_kick, st)
        if self.charges is not None:
            # the charge paint visits only the charged beads; the readout (with
            # the kick and the CSVR sums) visits all
            _lib.call("hpf_pic_step_list", self.pm._h, _lib.ptr(self.r), _lib.ptr(self.charges),
                      _lib.ptr(self.charged), self.charged.numel(), self.n,
                      float(self.elec_factor), _lib.ptr(self.f_elec), None, kick, st)

    # autotune the fused k-space pass's tile width in prime()
    TUNE_SPECTRAL_TILE = True

    def _tune_spectral_tile(self, reps=5):
        """Tile width of the fused k-space pass picked by timing the field
        step (CUDA events, `reps` steps per width after one warm-up) on the
        current positions; the fastest is kept.  Timings (us) are kept in
        `spectral_tile_timings`.  The forces are the same for every width."""
        widths = self.pm.spectral_tiles_allowed if self.pm.spectral == "fused" else []
        self.spectral_tile_timings = {}
        if len(widths) < 2:
            return
        st = _lib.stream_ptr()
        scratch = torch.zeros_like(self.field_sums)
        best = None
        for w in widths:
            self.pm.spectral_tile = w
            self._field(st, scratch)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                self._field(st, scratch)
            e1.record()
            e1.synchronize()
            t = e0.elapsed_time(e1) * 1000.0 / reps
            self.spectral_tile_timings[w] = t
            if best is None or t < best[0]:
                best = (t, w)
        self.pm.spectral_tile = best[1]

    def prime(self):
        """Bonded and slow forces at the initial positions (main.py:494-588).
        With the fused plan the bonded forces come from its deterministic
        gather (hpf_respa_forces), so that runs are bit-reproducible.  The
        k-space tile width is tuned first (`TUNE_SPECTRAL_TILE`)."""
        if self.TUNE_SPECTRAL_TILE and self.graph is None:
            self._tune_spectral_tile()
        st = _lib.stream_ptr()
        self._bonded(st, 0)
        if self.topo is not None:
            if self.plan is not None:
                _lib.call("hpf_respa_forces", self.plan, _lib.ptr(self.r), _lib.ptr(self.f_b),
                          _lib.ptr(self.box), None, _lib.ptr(self.err), st)
            else:
                self.f_b.copy_(self.f_bond)
                self.f_b.add_(self.f_angle)
                self.f_b.add_(self.f_dih)
        self._field(st, self.field_sums)
        if self.bias is not None:
            self._bias_forces()  # the bias of step 0 (main.py:691-724)
        if self.baro_args is not None:
            # the barostat reads the bonded virials of the last inner step
            for k, ws in ((0, self.ws_bond), (4, self.ws_angle)):
                self.bonded_out[k:k + 4].copy_(ws[:4])

    def _inner_fused(self, st):
        """First outer kick + all inner steps (+ the barostat's box update in
        the last block when coupled; positions follow in the next paint)."""
        fs = self._slow_forces()
        arr = (_lib.P * len(fs))(*[_lib.ptr(f) for f in fs])
        baro = self.baro_args is not None
        if self._paint_fused:
            _lib.call("hpf_respa_step_paint", self.plan, _lib.ptr(self.r), _lib.ptr(self.v),
                      _lib.ptr(self.f_b), arr, len(fs), self.mass, self.dt, self.respa,
                      _lib.ptr(self.box), _lib.ptr(self.dipoles), _lib.ptr(self.transfer),
                      _lib.ptr(self.bonded_out), self.pm._h, _lib.ptr(self.types),
                      _lib.ptr(self.charges),
                      _lib.ctypes.byref(self.baro_args) if baro else None,
                      _lib.ptr(self.field_sums) if baro else None,
                      _lib.ptr(self.randoms) if baro else None,
                      _lib.ptr(self.counter) if baro else None,
                      _lib.ptr(self.state) if baro else None, _lib.ptr(self.err), st)
            return
        _lib.call("hpf_respa_step", self.plan, _lib.ptr(self.r), _lib.ptr(self.v),
                  _lib.ptr(self.f_b), arr, len(fs), self.mass, self.dt, self.respa,
                  _lib.ptr(self.box), _lib.ptr(self.dipoles), _lib.ptr(self.transfer),
                  _lib.ptr(self.bonded_out), self.pm._h if baro else None,
                  _lib.ctypes.byref(self.baro_args) if baro else None,
                  _lib.ptr(self.field_sums) if baro else None,
                  _lib.ptr(self.randoms) if baro else None,
                  _lib.ptr(self.counter) if baro else None,
                  _lib.ptr(self.state) if baro else None, _lib.ptr(self.err), st)

    def _inner_unfused(self, st):
        fb, fa, fd = self._bonded_ptrs()
        self._outer_kick(st)
        for inner in range(self.respa):
            kicks = 1 if inner == 0 else 2
            _lib.call("hpf_inner_kick_drift", _lib.ptr(self.r), _lib.ptr(self.v), fb, fa, fd,
                      self.n, self.mass, self.dt, kicks, 1, _lib.ptr(self.box), st)
            self._bonded(st, 1 if inner == self.respa - 1 else 0)
        _lib.call("hpf_inner_kick_drift", _lib.ptr(self.r), _lib.ptr(self.v), fb, fa, fd, self.n,
                  self.mass, self.dt, 1, 0, None, st)

    def step(self):
        """One outer rRESPA step (launch sequence only; no host sync unless a
        bias is set)."""
        st = _lib.stream_ptr()
        self.step_count += 1
        if self.plan is not None:
            self._inner_fused(st)  # includes the barostat's box update
            self._outer_rest(st)
            return
        self._inner_unfused(st)
        if self.baro_args is not None:
            self.bonded_out[0:4].copy_(self.ws_bond[:4])
            self.bonded_out[4:8].copy_(self.ws_angle[:4])
            self._barostat(st)
        self._outer_rest(st, fused=False)

    def _outer_rest(self, st, fused=True):
        """The part of the outer step after the inner loop: field forces with
        the second outer half kick (and the CSVR sums) fused into the last
        readout, then the thermostat's scaling."""
        scale = None
        painted = fused and self._paint_fused
        if fused and self.baro_args is not None:
            if self.baro_mode == 0:
                # alpha, applied in the paint, or after a fused paint by the
                # density readout as it reads the positions
                scale = self.state.data_ptr() + 12 * 8
            else:
                # semi-isotropic (mode 1): a position kernel of its own
                _lib.call("hpf_scr_scale_positions", _lib.ptr(self.r), self.n,
                          _lib.ptr(self.state), self.baro_mode, st)
        thermo = self.thermo_args is not None
        if self.bias is not None:
            # the bias needs the new field forces before the second kick:
            # field step without the fused kick, the bias on the host, then
            # the kick with every slow force (and the CSVR in the same pass)
            self._field(st, self.field_sums, pos_scale=scale, painted=painted)
            self._bias_forces()
            st = _lib.stream_ptr()
            if thermo:
                self._thermostat(st, kick=True)
            else:
                self._outer_kick(st)
            return
        self._field(st, self.field_sums, pos_scale=scale, kick=self._kick_args(thermo),
                    painted=painted)
        if thermo:
            _lib.call("hpf_csvr_scale", _lib.ptr(self.v), _lib.ptr(self.group), self.n,
                      _lib.ptr(self.state), int(self.thermo_args.remove_com), st)

    def capture(self, split=False):
        """Record one outer step in a CUDA graph (after a warm-up step).

        With split=True (fused inner loop only) the step is recorded as two
        graphs replayed back to back -- `graph_inner` (the fused rRESPA kernel)
        and `graph_field` (field step, kick, thermostat) -- so that a caller
        can put timing events between them."""
        if self.bias is not None:
            raise RuntimeError("a bias runs on the host every step: run() steps eagerly")
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.step()
        torch.cuda.current_stream(self.device).wait_stream(s)
        torch.cuda.synchronize(self.device)
        self.graph_inner = self.graph_field = None
        if split and self.plan is not None:
            gi, gf = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
            with torch.cuda.graph(gi):
                self._inner_fused(_lib.stream_ptr())
            with torch.cuda.graph(gf, pool=gi.pool()):
                self._outer_rest(_lib.stream_ptr())
            self.graph_inner, self.graph_field = gi, gf
            self.graph = None
            return gi, gf
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step()
        self.graph = g
        return g

    def replay(self):
        """One outer step from the captured graph(s)."""
        if self.graph_inner is not None:
            self.graph_inner.replay()
            self.graph_field.replay()
        else:
            self.graph.replay()

    def run(self, steps):
        """`steps` outer steps (graph replays once captured); with
        resort_every > 0 the beads are re-sorted by mesh cell after every
        resort_every-th step."""
        for _ in range(steps):
            if self.graph is not None or self.graph_inner is not None:
                self.replay()
            else:
                self.step()
            self.steps_run += 1
            if self.resort_every and self.steps_run % self.resort_every == 0:
                self.resort()

    def run_host(self, r_in, v_in, r_out, steps=1):
        """`steps` outer steps, each from a host-side state: positions and
        velocities are copied in from the page-locked host tensors r_in, v_in
        before the step and the positions copied out to r_out after it
        (stream-ordered DMA copies; the CPU-GPU link moves about 200 GB/s each
        way, and a copy kernel reading the mapped host memory was no faster).
        Host tensors are (N, 3) float32 in this object's bead order
        (`in_input_order` maps back)."""
        for t in (r_in, v_in, r_out):
            if t.device.type != "cpu" or not t.is_pinned() or t.dtype != torch.float32 \
                    or tuple(t.shape) != (self.n, 3):
                raise ValueError("run_host: page-locked float32 (N, 3) host tensors")
        for _ in range(steps):
            self.r.copy_(r_in, non_blocking=True)
            self.v.copy_(v_in, non_blocking=True)
            self.run(1)
            r_out.copy_(self.r, non_blocking=True)

    # ------------------------------------------------------------------
    def energies(self):
        """(bond, angle, dihedral) energies of the last inner step (FP64)."""
        if self.plan is not None:
            o = self.bonded_out.cpu().numpy()
            return [float(o[0]), float(o[4]), float(o[8])]
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
