"""ctypes wrapper over the C restatement of HyMD's Fortran bonded kernels
(test infrastructure only).

orc_bonds / orc_angles / orc_dihedrals follow hymd/compute_bond_forces.f90,
hymd/compute_angle_forces.f90, hymd/compute_dihedral_forces.f90 and
hymd/dipole_reconstruction.f90 (see bonded_oracle_impl.h for line-level notes).
`precision="single"` mirrors cbf/caf/cdf (real(4) storage), "double" mirrors
cbf_d/caf_d/cdf_d.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "libbonded_oracle.so")
        src = os.path.join(_HERE, "bonded_oracle_impl.h")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            subprocess.check_call(["make", "-s", "-C", _HERE, "libbonded_oracle.so"])
        _LIB = ctypes.CDLL(path)
    return _LIB


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _idx(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int64).reshape(-1))


def _real(precision):
    return (np.float32, "_f32") if precision == "single" else (np.float64, "_f64")


def compute_bond_forces(f, r, box, a, b, r0, k, precision="single"):
    """cbf(f, r, box, a, b, r0, k) -> (energy, bond_pr); f overwritten."""
    dt, sfx = _real(precision)
    assert f.dtype == dt and r.dtype == dt and f.flags.c_contiguous
    r = np.ascontiguousarray(r)
    a, b = _idx(a), _idx(b)
    r0 = np.ascontiguousarray(r0, dtype=np.float64)
    k = np.ascontiguousarray(k, dtype=np.float64)
    box = np.ascontiguousarray(box, dtype=np.float64)
    e = ctypes.c_double(0.0)
    pr = np.zeros(3, dtype=dt)
    getattr(_lib(), "orc_bonds" + sfx)(
        _p(f), _p(r), ctypes.c_int64(len(r)), _p(box), _p(a), _p(b), _p(r0), _p(k),
        ctypes.c_int64(len(a)), ctypes.byref(e), _p(pr))
    return e.value, pr


def compute_angle_forces(f, r, box, a, b, c, t0, k, precision="single"):
    """caf(f, r, box, a, b, c, t0, k) -> (energy, angle_pr); f overwritten."""
    dt, sfx = _real(precision)
    assert f.dtype == dt and r.dtype == dt and f.flags.c_contiguous
    r = np.ascontiguousarray(r)
    a, b, c = _idx(a), _idx(b), _idx(c)
    t0 = np.ascontiguousarray(t0, dtype=np.float64)
    k = np.ascontiguousarray(k, dtype=np.float64)
    box = np.ascontiguousarray(box, dtype=np.float64)
    e = ctypes.c_double(0.0)
    pr = np.zeros(3, dtype=dt)
    getattr(_lib(), "orc_angles" + sfx)(
        _p(f), _p(r), ctypes.c_int64(len(r)), _p(box), _p(a), _p(b), _p(c), _p(t0), _p(k),
        ctypes.c_int64(len(a)), ctypes.byref(e), _p(pr))
    return e.value, pr


def compute_dihedral_forces(f, r, dipoles, transfer, box, a, b, c, d, coeff, dtype,
                            last, dipole_flag, precision="single"):
    """cdf(...) -> energy; f, dipoles (D,4,3), transfer (D,6,3,3) overwritten."""
    dt, sfx = _real(precision)
    assert f.dtype == dt and dipoles.dtype == dt and transfer.dtype == dt
    assert f.flags.c_contiguous and dipoles.flags.c_contiguous and transfer.flags.c_contiguous
    r = np.ascontiguousarray(r)
    a, b, c, d = _idx(a), _idx(b), _idx(c), _idx(d)
    coeff = np.ascontiguousarray(np.asarray(coeff).reshape(len(a), 6, 5), dtype=np.float32)
    dtype_, last = _idx(dtype), _idx(last)
    box = np.ascontiguousarray(box, dtype=np.float64)
    e = ctypes.c_double(0.0)
    getattr(_lib(), "orc_dihedrals" + sfx)(
        _p(f), _p(r), ctypes.c_int64(len(r)), _p(dipoles), _p(transfer), _p(box),
        _p(a), _p(b), _p(c), _p(d), _p(coeff), _p(dtype_), _p(last),
        ctypes.c_int64(len(a)), ctypes.c_int(int(dipole_flag)), ctypes.byref(e))
    return e.value


def dipole_forces_redistribution(n_particles, f_dipoles, trans_matrices, a, b, c, d,
                                 type_array, last_bb):
    """hymd/force.py:855-877 in FP64: map dipole pseudo-charge forces to beads."""
    out = np.zeros((n_particles, 3), dtype=np.float64)
    fd_all = np.asarray(f_dipoles, dtype=np.float64).reshape(-1, 4, 3)
    tm_all = np.asarray(trans_matrices, dtype=np.float64).reshape(-1, 6, 3, 3)
    for i, j, k, l, fd, m, t, last in zip(a, b, c, d, fd_all, tm_all, type_array, last_bb):
        if t == 1:
            s = fd[0] + fd[1]
            df = fd[0] - fd[1]
            out[i] += m[0] @ df
            out[j] += m[1] @ df + 0.5 * s
            out[k] += m[2] @ df + 0.5 * s
            if last == 1:
                s = fd[2] + fd[3]
                df = fd[2] - fd[3]
                out[j] += m[3] @ df
                out[k] += m[4] @ df + 0.5 * s
                out[l] += m[5] @ df + 0.5 * s
    return out
