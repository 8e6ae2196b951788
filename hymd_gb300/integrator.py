"""Velocity-Verlet pieces -- drop-in for hymd/integrator.py:9-73.

Both functions return new tensors (the reference returns new arrays) and run
in libhpf_gb300.so with the reference's FP32 rounding sequence:
    v_new = v + (0.5 * dt) * a        x_new = x + dt * v
"""
import torch

from . import _lib


def integrate_velocity(velocities, accelerations, time_step):
    v = _lib.require_cuda(velocities, "velocities", torch.float32).clone()
    a = _lib.require_cuda(accelerations, "accelerations", torch.float32, tuple(v.shape))
    arr = (_lib.P * 1)(_lib.ptr(a))
    _lib.call("hpf_kick", _lib.ptr(v), arr, 1, v.shape[0], 1.0, float(time_step), _lib.stream_ptr())
    return v


def integrate_position(positions, velocities, time_step):
    r = _lib.require_cuda(positions, "positions", torch.float32).clone()
    v = _lib.require_cuda(velocities, "velocities", torch.float32, tuple(r.shape)).clone()
    _lib.call("hpf_inner_kick_drift", _lib.ptr(r), _lib.ptr(v), None, None, None, r.shape[0], 1.0,
              float(time_step), 0, 1, None, _lib.stream_ptr())
    return r
