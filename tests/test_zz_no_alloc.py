"""The allocation-free paint (hpf_paint_static) against the context paint
(hpf_paint): the same per-type densities, bit for bit, on two calls in a row
with different particles -- the second call shows that the static scratch is
cleared between calls.  Kept last in collection order so that it also runs
after every other test has used the library.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _particles(seed, n, T, box):
    rng = np.random.default_rng(seed)
    r = (rng.uniform(0, 1, (n, 3)) * box).astype(np.float32)
    r[: n // 4] = np.mod(box / 2 + rng.normal(0, 0.5, (n // 4, 3)), box).astype(np.float32)
    types = rng.integers(0, T, n).astype(np.int32)
    return torch.as_tensor(r, device="cuda"), torch.as_tensor(types, device="cuda")


@pytest.mark.parametrize("mesh,box", [((32, 32, 32), (6.0, 6.5, 7.0)),
                                      ((25, 21, 18), (5.0, 4.0, 3.7))])
def test_static_paint_matches_context_paint(mesh, box):
    from hymd_gb300 import _lib
    from hymd_gb300.field import ParticleMesh, paint_static

    T = 3
    masses = [72.0, 54.0, 1.5]
    box = np.asarray(box, np.float64)
    pm = ParticleMesh(mesh, box, T)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    for call, seed in enumerate((11, 12)):
        r, ty = _particles(seed, 20000 + 5000 * call, T, box)
        ref = pm.real_field(T)
        _lib.call("hpf_paint", pm._h, _lib.ptr(r), _lib.ptr(ty), r.shape[0], _lib.dvec(masses),
                  _lib.ptr(ref), _lib.stream_ptr())
        out = paint_static(r, ty, masses, mesh, box, err=err)
        torch.cuda.synchronize()
        assert torch.equal(out, ref), f"call {call}: static paint differs from hpf_paint"
        # mass conservation as a sanity check (sum phi dV = sum of masses)
        dV = float(np.prod(box)) / float(np.prod(mesh))
        tot = float(out.double().sum()) * dV
        want = float(sum(masses[t] * int((ty == t).sum()) for t in range(T)))
        assert abs(tot - want) <= 1e-5 * want
    assert int(err.item()) == 0
    pm.check_errors()


def test_static_paint_rejects_oversized_mesh():
    from hymd_gb300 import _lib
    from hymd_gb300.field import paint_static

    r, ty = _particles(3, 100, 2, np.array([5.0, 5.0, 5.0]))
    with pytest.raises(_lib.HPFError, match="HPF_ERR_SCRATCH_LIMIT"):
        paint_static(r, ty, [1.0, 1.0], (128, 128, 128), (5.0, 5.0, 5.0))


def test_static_paint_into_offset_view():
    """Destinations that start 4 bytes past a 16-byte boundary (a contiguous
    view into a larger buffer) take the scalar store path: same grids, bit for
    bit, from both paints."""
    from hymd_gb300 import _lib
    from hymd_gb300.field import ParticleMesh, paint_static

    T, mesh = 2, (32, 32, 32)
    box = np.array([6.0, 6.0, 6.0])
    masses = [72.0, 36.0]
    M = int(np.prod(mesh))
    r, ty = _particles(21, 8000, T, box)
    ref = paint_static(r, ty, masses, mesh, box)
    buf = torch.zeros(T * M + 1, dtype=torch.float32, device="cuda")
    view = buf[1:].view(T, *mesh)
    assert view.data_ptr() % 16 == 4
    paint_static(r, ty, masses, mesh, box, out=view)
    pm = ParticleMesh(mesh, box, T)
    buf2 = torch.zeros(T * M + 1, dtype=torch.float32, device="cuda")
    view2 = buf2[1:].view(T, *mesh)
    _lib.call("hpf_paint", pm._h, _lib.ptr(r), _lib.ptr(ty), r.shape[0], _lib.dvec(masses),
              _lib.ptr(view2), _lib.stream_ptr())
    torch.cuda.synchronize()
    assert torch.equal(view, ref) and torch.equal(view2, ref)
    assert float(buf[0]) == 0.0 and float(buf2[0]) == 0.0
    pm.check_errors()
