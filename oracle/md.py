"""Oracle rRESPA step (test infrastructure only): hymd/main.py:802-887,
975-1004 and 1143-1169 on the FP64 field oracle and the FP32 bonded oracle,
with the FP32 state updates of hymd/integrator.py:9-73."""
import numpy as np

from . import bonded
from . import field as of


def _kick(v, f, mass, dt):
    # integrate_velocity(v, f / mass, dt) in float32, as the reference arrays are
    return (v + np.float32(0.5 * dt) * (f.astype(np.float32) / np.float32(mass))).astype(np.float32)


def field_forces(r, types, cfg, functional):
    out = of.update_field(r.astype(np.float64), types, cfg.n_types, cfg.mesh(), cfg.box(),
                          cfg.m or [1.0] * cfg.n_types, functional, cfg.sigma)
    return of.compute_field_force(out["force_mesh"], r.astype(np.float64), types, cfg.n_types,
                                  cfg.mesh(), cfg.box()).astype(np.float32)


def bonded_forces(r, topo, box):
    (b2a, b2b, b2r, b2k, b3a, b3b, b3c, b3t, b3k, *_rest) = topo
    fb = np.zeros_like(r)
    fa = np.zeros_like(r)
    if len(b2a):
        bonded.compute_bond_forces(fb, r, box, b2a, b2b, b2r, b2k)
    if len(b3a):
        bonded.compute_angle_forces(fa, r, box, b3a, b3b, b3c, b3t, b3k)
    return fb, fa


def respa_step(r, v, f_field, types, topo, cfg, functional, bias=None, f_bias=None, step=1):
    """One outer step; returns (r, v, f_field), or (r, v, f_field, f_bias)
    with a bias: `bias(step, r, current_forces)` returns the bias force of the
    positions after the field update (hymd/main.py:1097-1141), and f_bias
    (that of the previous step) is kicked with the field force in both outer
    half kicks (main.py:808-812, 1150-1154)."""
    box = cfg.box()
    dt = cfg.time_step
    mass = cfg.mass
    v = _kick(v, f_field, mass, cfg.respa_inner * dt)
    if bias is not None:
        v = _kick(v, f_bias, mass, cfg.respa_inner * dt)
    fb, fa = bonded_forces(r, topo, box)
    for _ in range(cfg.respa_inner):
        v = _kick(v, (fb + fa).astype(np.float32), mass, dt)
        r = (r + np.float32(dt) * v).astype(np.float32)
        r = np.mod(r, box.astype(np.float32)).astype(np.float32)
        fb, fa = bonded_forces(r, topo, box)
        v = _kick(v, (fb + fa).astype(np.float32), mass, dt)
    f_field = field_forces(r, types, cfg, functional)
    if bias is not None:
        f_bias = np.asarray(bias(step, r, f_field + fb + fa), np.float32)
    v = _kick(v, f_field, mass, cfg.respa_inner * dt)
    if bias is not None:
        v = _kick(v, f_bias, mass, cfg.respa_inner * dt)
        return r, v, f_field, f_bias
    return r, v, f_field
