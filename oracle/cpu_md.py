"""FP32 multi-core CPU restatement of one HyMD outer rRESPA step -- TEST
INFRASTRUCTURE ONLY (the timed CPU baseline of bench.py; never on the
product path).

The reference's own CPU path (pmesh/pfft + f2py Fortran under mpirun) cannot
be built here or on the GPU machine (no gfortran, MPI, pmesh or pfft; numpy 2 has
no numpy.distutils for its setup.py), so this restates it, in the reference's
default float32 and in its order of operations, on all host cores:

  outer half kick with the slow forces          hymd/main.py:802-827
  respa_inner x [kick, drift, wrap, bonded
                 forces (cbf, caf, cdf), kick]   hymd/main.py:830-887
  update_field: per type paint, r2c, H, c2r;
    v_ext; per type r2c, H, 3 x (-i k_d, c2r)   hymd/field.py:570-616
  compute_field_force (readout)                 hymd/field.py:197-200
  update_field_force_q (PIC_Spectral)           hymd/field.py:356-403
  second outer half kick                        hymd/main.py:1143-1169
  CSVR thermostat                               hymd/thermostat.py:111-219

Paint, readout, the k-space maps, v_ext and the kick/drift run in
oracle/cpu_field.c (OpenMP over the cores, in place of the reference's MPI
ranks); the transforms are scipy.fft's with `workers` threads; the bonded
terms are the C restatement of the Fortran kernels (oracle/bonded.py; serial,
as each Fortran call is per rank).
"""
import ctypes
import os
import subprocess

import numpy as np

from . import bonded
from . import coupling

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "libcpu_field.so")
        src = os.path.join(_HERE, "cpu_field.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            subprocess.check_call(["make", "-s", "-C", _HERE, "libcpu_field.so"])
        L = ctypes.CDLL(path)
        P, I64, I, D = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
        L.cpu_paint.argtypes = [P, P, P, P, I64, I, I, I, I, P, P]
        L.cpu_readout.argtypes = [P, P, P, P, I64, I, I, I, I, P, P]
        L.cpu_kmap.argtypes = [P, P, I, I, I, P, I, I, D, D]
        L.cpu_vext.argtypes = [P, I, I64, P, D, P]
        L.cpu_kick_drift.argtypes = [P, P, P, I, I64, D, D, D, P, I]
        L.cpu_threads.restype = I
        _LIB = L
    return _LIB


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def threads():
    return int(lib().cpu_threads())


class CpuStep:
    """State and one outer step of a system built by hymd_gb300.systems
    (positions, velocities, types, topology, config[, charges]), with the
    quadratic functional (Q, b) of its Hamiltonian."""

    def __init__(self, system, Q, b, workers=None, thermostat=True, seed=0):
        import scipy.fft  # noqa: F401  (threaded transforms)
        self.cfg = cfg = system["config"]
        self.r = np.ascontiguousarray(system["positions"], np.float32).copy()
        self.v = np.ascontiguousarray(system["velocities"], np.float32).copy()
        self.types = np.ascontiguousarray(system["types"], np.int32)
        self.n = len(self.r)
        self.T = int(cfg.n_types)
        self.mesh = tuple(int(x) for x in cfg.mesh())
        self.box = np.ascontiguousarray(cfg.box(), np.float64)
        self.M = int(np.prod(self.mesh))
        self.dV = float(np.prod(self.box)) / self.M
        self.Q = np.ascontiguousarray(Q, np.float64)
        self.b = np.asarray(b, np.float64)
        self.m = np.asarray(list(cfg.m) if cfg.m else [1.0] * self.T, np.float64)
        self.workers = workers or os.cpu_count() or 1
        topo = system.get("topology")
        self.topo = topo
        q = system.get("charges")
        self.q = None if q is None else np.ascontiguousarray(q, np.float32)
        self.elec = None
        if self.q is not None and np.any(self.q):
            self.elec = 4.0 * np.pi * cfg.coulomb_constant / cfg.dielectric_const
        nh = self.mesh[2] // 2 + 1
        self.spec = np.empty((self.mesh[0], self.mesh[1], nh), np.complex64)
        self.spec2 = np.empty_like(self.spec)
        self.phi = np.empty((self.T,) + self.mesh, np.float32)
        self.fmesh = np.empty((self.T, 3) + self.mesh, np.float32)
        self.emesh = np.empty((3,) + self.mesh, np.float32)
        self.vtmp = np.empty(self.mesh, np.float32)
        z = lambda: np.zeros((self.n, 3), np.float32)  # noqa: E731
        self.f_field, self.f_elec, self.f_b = z(), z(), z()
        self._fb, self._fa, self._fd = z(), z(), z()
        nd = 0 if topo is None else len(topo[9])
        self.dip = np.zeros((max(nd, 1), 4, 3), np.float32)
        self.tr = np.zeros((max(nd, 1), 6, 3, 3), np.float32)
        self.thermostat = thermostat and bool(cfg.target_temperature)
        self.rng = np.random.default_rng(seed)
        self.bonded_forces(0)
        self.field_forces()

    # ---- transforms (r2c / M, c2r unnormalised) ----------------------------
    def _r2c(self, grid, out):
        import scipy.fft as sf
        out[...] = sf.rfftn(grid, norm="forward", workers=self.workers)
        return out

    def _c2r(self, spec, out):
        import scipy.fft as sf
        out[...] = sf.irfftn(spec, s=self.mesh, norm="forward", workers=self.workers)
        return out

    def _kmap(self, src, dst, mode, d=0, c=0.0):
        L = lib()
        n0, n1, n2 = self.mesh
        L.cpu_kmap(_p(src), _p(dst), n0, n1, n2, _p(self.box), mode, d, float(self.cfg.sigma),
                   float(c))

    # ---- forces ---------------------------------------------------------------
    def field_forces(self):
        L = lib()
        n0, n1, n2 = self.mesh
        gscale = (self.m / self.dV).astype(np.float32)
        L.cpu_paint(_p(self.r), _p(self.types), None, _p(gscale), self.n, self.T, n0, n1, n2,
                    _p(self.box), _p(self.phi))
        for t in range(self.T):
            self._r2c(self.phi[t], self.spec)
            self._kmap(self.spec, self.spec, 0)
            self._c2r(self.spec, self.phi[t])
        for t in range(self.T):
            L.cpu_vext(_p(self.phi), self.T, self.M, _p(np.ascontiguousarray(self.Q[t])),
                       float(self.b[t]), _p(self.vtmp))
            self._r2c(self.vtmp, self.spec)
            self._kmap(self.spec, self.spec, 0)
            for d in range(3):
                self._kmap(self.spec, self.spec2, 1, d)
                self._c2r(self.spec2, self.fmesh[t, d])
        L.cpu_readout(_p(self.fmesh), _p(self.r), _p(self.types), None, self.n, 3, n0, n1, n2,
                      _p(self.box), _p(self.f_field))
        if self.elec is not None:
            one = np.array([1.0 / self.dV], np.float32)
            L.cpu_paint(_p(self.r), None, _p(self.q), _p(one), self.n, 1, n0, n1, n2,
                        _p(self.box), _p(self.vtmp))
            self._r2c(self.vtmp, self.spec)
            self._kmap(self.spec, self.spec, 0)
            self._kmap(self.spec, self.spec, 2, c=self.elec)
            self._c2r(self.spec, self.vtmp)  # psi (kept by the reference for the energy)
            for d in range(3):
                self._kmap(self.spec, self.spec2, 1, d)
                self._c2r(self.spec2, self.emesh[d])
            L.cpu_readout(_p(self.emesh), _p(self.r), None, _p(self.q), self.n, 3, n0, n1, n2,
                          _p(self.box), _p(self.f_elec))

    def bonded_forces(self, dipole_flag):
        t = self.topo
        if t is None:
            return
        (b2a, b2b, b2r, b2k, b3a, b3b, b3c, b3t, b3k, b4a, b4b, b4c, b4d, b4coeff, b4type,
         b4last) = t
        box = self.box
        if len(b2a):
            bonded.compute_bond_forces(self._fb, self.r, box, b2a, b2b, b2r, b2k)
        if len(b3a):
            bonded.compute_angle_forces(self._fa, self.r, box, b3a, b3b, b3c, b3t, b3k)
        if len(b4a):
            bonded.compute_dihedral_forces(self._fd, self.r, self.dip, self.tr, box, b4a, b4b,
                                           b4c, b4d, b4coeff, b4type, b4last, dipole_flag)
        np.add(self._fb, self._fa, out=self.f_b)
        np.add(self.f_b, self._fd, out=self.f_b)

    # ---- the step -------------------------------------------------------------
    def _kick(self, forces, h, drift=False):
        arr = (ctypes.c_void_p * len(forces))(*[f.ctypes.data for f in forces])
        lib().cpu_kick_drift(_p(self.r), _p(self.v), arr, len(forces), self.n,
                             float(self.cfg.mass), float(h), float(self.cfg.time_step),
                             _p(self.box), int(drift))

    def slow(self):
        return [self.f_field] + ([self.f_elec] if self.elec is not None else [])

    def step(self):
        cfg = self.cfg
        dt, k = float(cfg.time_step), int(cfg.respa_inner)
        self._kick(self.slow(), 0.5 * dt * k)
        for inner in range(k):
            self._kick([self.f_b], 0.5 * dt, drift=True)
            self.bonded_forces(1 if inner == k - 1 else 0)
            self._kick([self.f_b], 0.5 * dt)
        self.field_forces()
        self._kick(self.slow(), 0.5 * dt * k)
        if self.thermostat:
            n = self.n
            draws = [self.rng.normal(), self.rng.chisquare(3 * n - 1)]
            v, _ = coupling.csvr(self.v, np.zeros(n, np.int32), 1, float(cfg.mass),
                                 float(cfg.target_temperature), dt * k, float(cfg.tau), draws)
            self.v[...] = v
