"""Trajectory and observable output of a device MD run every n_print steps
(the output block of hymd/main.py:1323-1442) without stalling the device.

`record(step)` enqueues, on the run's stream, the FP64 energy and pressure
sums of the current positions (hpf_energy_fp64), the kinetic sum, the
bonded energies and virials of the last inner step, the thermostat work and
the box, and device-to-device snapshots of positions, velocities and the
total force (field + bonded + electrostatic, as main.py:1403-1413 sums them)
in the caller's bead order.  A side stream then copies the slot to
page-locked host memory while the next steps run, and (threaded=True, the
default) a writer thread passes each frame to file_io.store_data as soon as
its copy has finished, so that neither the device nor the thread launching
the steps waits for the host-side write (numpy releases the interpreter lock
in its copies and dot products).  Without the thread, `drain()` writes the
frames whose copies have finished.  `close()` waits for the rest.  Slots are
reused round-robin: with `depth` slots in flight a record() waits only if
the oldest snapshot has not been written yet.

Per frame it costs one FP64 energy evaluation and ~3 copies of N x 3 floats
on the device; the step graph itself is untouched.
"""
import collections
import queue
import threading

import numpy as np
import torch

from . import _lib
from .field import decode_energy_sums
from .file_io import store_data
from .pressure import pressure_vector


class _Slot:
    def __init__(self, n, dev, need_v, need_f):
        z = lambda: torch.empty((n, 3), dtype=torch.float32, device=dev)  # noqa: E731
        h = lambda: torch.empty((n, 3), dtype=torch.float32, pin_memory=True)  # noqa: E731
        self.r, self.hr = z(), h()
        self.v, self.hv = (z(), h()) if need_v else (None, None)
        self.f, self.hf = (z(), h()) if need_f else (None, None)
        self.sums = torch.zeros(32, dtype=torch.float64, device=dev)
        self.misc = torch.zeros(32, dtype=torch.float64, device=dev)
        self.hsums = torch.empty(32, dtype=torch.float64, pin_memory=True)
        self.hmisc = torch.empty(32, dtype=torch.float64, pin_memory=True)
        self.done = torch.cuda.Event()
        self.written = threading.Event()
        self.written.set()
        self.step = self.frame = None


class TrajectoryRecorder:
    """Asynchronous store_data feed for a RespaMD.

    md: the RespaMD; out: a file_io.OutDataset on which store_static has been
    called; hamiltonian: the run's functional; indices: the global index of
    each bead in the caller's order (default 0..N-1); pressure: compute the
    18-vector (default: config.pressure or a barostat, as main.py does)."""

    def __init__(self, md, out, hamiltonian, indices=None, velocity_out=False, force_out=False,
                 pressure=None, depth=3, dump_per_particle=False, threaded=True):
        self.md = md
        self.out = out
        self.cfg = cfg = md.config
        self.n = md.n
        self.indices = np.arange(md.n) if indices is None else np.asarray(indices)
        self.velocity_out = velocity_out
        self.force_out = force_out
        self.dump_per_particle = dump_per_particle
        self.charge_out = md.charges is not None
        self.Q, self.b, self.c, self.sigma = md.pm.set_functional(hamiltonian)
        self.pressure = bool(cfg.pressure or cfg.barostat) if pressure is None else pressure
        self.type_charges = (_lib.dvec([float(x) for x in cfg.type_charges])
                             if self.charge_out and cfg.type_charges is not None else None)
        self.elec_factor = (cfg.coulomb_constant / cfg.dielectric_const) if self.charge_out else 0.0
        dev = md.device
        # the kinetic sum needs v on the device even when v is not written
        self.slots = [_Slot(md.n, dev, True, force_out) for _ in range(max(1, depth))]
        self.next = 0
        self.pending = collections.deque()
        self.ws = _lib.new_workspace(dev)
        self.copy_stream = torch.cuda.Stream(device=dev)
        self.written = 0
        self._error = None
        self._queue = queue.Queue() if threaded else None
        self._thread = None
        if threaded:
            self._thread = threading.Thread(target=self._writer, name="hpf-trajectory",
                                            daemon=True)
            self._thread.start()

    def _writer(self):
        while True:
            s = self._queue.get()
            if s is None:
                self._queue.task_done()
                return
            try:
                if self._error is None:
                    self._write(s, block=True)
            except BaseException as e:  # surfaced by the next record/drain/close
                self._error = e
            finally:
                s.written.set()
                self._queue.task_done()

    def _check(self):
        if self._error is not None:
            e, self._error = self._error, None
            raise RuntimeError("trajectory writer failed") from e

    def _free(self):
        self._check()
        if self._queue is not None and self._thread is None:
            raise RuntimeError("TrajectoryRecorder.record() after close()")
        s = self.slots[self.next]
        if self._queue is not None:
            s.written.wait()  # the writer thread is done with this slot
            self._check()
        elif s.step is not None:  # still holds a snapshot: write it first
            while self.pending and self.pending[0] is not s:
                self._write(self.pending.popleft(), block=True)
            if self.pending:
                self._write(self.pending.popleft(), block=True)
        self.next = (self.next + 1) % len(self.slots)
        return s

    def record(self, step, frame=None):
        """Snapshot the current state for output step `step` (frame
        step // n_print unless given); returns without waiting for the
        device."""
        md = self.md
        s = self._free()
        st = _lib.stream_ptr()
        _lib.call("hpf_energy_fp64", md.pm._h, _lib.ptr(md.r), _lib.ptr(md.types), md.n,
                  md.masses, _lib.ptr(md.charges) if self.charge_out else None,
                  self.type_charges, float(self.elec_factor), _lib.ptr(s.sums), st)
        _lib.call("hpf_sum_v2", _lib.ptr(md.v), md.n, _lib.ptr(self.ws), st)
        s.misc.zero_()
        s.misc[0:1].copy_(self.ws[0:1])
        if md.plan is not None:
            s.misc[1:10].copy_(md.bonded_out[0:9])
        else:
            s.misc[1:5].copy_(md.ws_bond[0:4])
            s.misc[5:9].copy_(md.ws_angle[0:4])
            s.misc[9:10].copy_(md.ws_dih[0:1])
        s.misc[10:12].copy_(md.state[8:10])
        s.misc[12:15].copy_(md.box)
        perm = md.perm

        def put(dst, src):
            if perm is None:
                dst.copy_(src)
            else:
                dst.index_copy_(0, perm, src)

        put(s.r, md.r)
        put(s.v, md.v)
        if self.force_out:
            f = md.f_field + md.f_b
            if md.f_elec is not None:
                f = f + md.f_elec
            put(s.f, f)
        ready = torch.cuda.Event()
        ready.record()
        with torch.cuda.stream(self.copy_stream):
            self.copy_stream.wait_event(ready)
            for d, h in ((s.r, s.hr), (s.v, s.hv), (s.f, s.hf), (s.sums, s.hsums),
                         (s.misc, s.hmisc)):
                if d is not None:
                    h.copy_(d, non_blocking=True)
            s.done.record(self.copy_stream)
        # keep the device tensors alive for the copy stream
        for d in (s.r, s.v, s.f, s.sums, s.misc):
            if d is not None:
                d.record_stream(self.copy_stream)
        s.step = int(step)
        s.frame = int(step) // int(self.cfg.n_print) if frame is None else int(frame)
        if self._queue is not None:
            s.written.clear()
            self._queue.put(s)
        else:
            self.pending.append(s)

    def drain(self, block=False):
        """Write the snapshots whose host copies are complete (all of them
        with block=True), oldest first.  Returns the number written.  With
        the writer thread the frames are written as they arrive: drain()
        only waits for them (block=True) and returns 0."""
        if self._queue is not None:
            if block:
                self._queue.join()
            self._check()
            return 0
        k = 0
        while self.pending:
            s = self.pending[0]
            if not block and not s.done.query():
                break
            self._write(self.pending.popleft(), block=True)
            k += 1
        return k

    def close(self):
        self.drain(block=True)
        if self._thread is not None:
            self._queue.put(None)
            self._thread.join()
            self._thread = None

    def _write(self, s, block):
        s.done.synchronize()
        cfg = self.cfg
        m = s.hmisc.numpy()
        box = m[12:15].copy()
        V = float(np.prod(box))
        e = decode_energy_sums(s.hsums.numpy(), self.Q, self.b, self.c, self.sigma, V,
                               int(cfg.n_types))
        ke = 0.5 * float(cfg.mass) * float(m[0])
        self_energy = float(cfg.self_energy or 0.0)
        wq = 0.5 * V * e["Eq"] - self_energy if self.charge_out else 0.0
        temperature = (2.0 / 3.0) * ke / (cfg.gas_constant * cfg.n_particles)
        pressure = (pressure_vector(e, ke, m[2:5], m[6:9],
                                    self_energy if self.charge_out else None)
                    if self.pressure else 0.0)
        cfg.thermostat_work = float(m[10] + m[11])
        store_data(self.out, s.step, s.frame, self.indices, s.hr.numpy(),
                   s.hv.numpy(), s.hf.numpy() if s.hf is not None else np.zeros((self.n, 3)),
                   box, temperature, pressure, ke, float(m[1]), float(m[5]), float(m[9]),
                   float(e["W"]), wq, 0.0, cfg.respa_inner * cfg.time_step, cfg,
                   velocity_out=self.velocity_out, force_out=self.force_out,
                   charge_out=self.charge_out, plumed_out=False,
                   dump_per_particle=self.dump_per_particle)
        s.step = s.frame = None
        self.written += 1
