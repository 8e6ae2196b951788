"""A one-rank numpy stand-in for the parts of pmesh that HyMD's field path calls.

Test infrastructure only: `make_field_ref.py` passes this module as the
`pmesh` argument of the reference's unmodified `initialize_pm`
(hymd/field.py:10-149), so that the reference's own `update_field`,
`compute_field_force`, `update_field_force_q`, `update_field_force_q_GPE`,
`compute_field_and_kinetic_energy`, `comp_laplacian`, `comp_pressure` and the
SCR barostat run in this container, where pmesh/pfft are not installed.

pmesh is third-party (rainwoodman/pmesh, unpinned in HyMD's requirements.txt)
and is not vendored with the reference.  What is restated here is the subset
of its published behaviour that HyMD relies on, with the conventions the
FP64 oracle states (oracle/field.py):

  * ParticleMesh(Nmesh, BoxSize, dtype, comm): a periodic mesh of Nmesh[d]
    nodes at x = i * BoxSize[d] / Nmesh[d].
  * paint(pos, mass, layout, out): cloud-in-cell deposit of `mass` (scalar or
    per particle) onto the 8 nodes around each particle, weights
    (1 - |s - i|) per axis with s = x * Nmesh / BoxSize, periodic; the field
    holds sum(mass * W), not divided by the cell volume (the reference divides
    by volume_per_cell itself, field.py:574-575).
  * RealField.readout(pos, layout): the same 8-node weights, gathered.
  * RealField.r2c(out): forward real-to-complex transform normalised by 1/M;
    ComplexField.c2r(out): unnormalised inverse, so c2r(r2c(f)) == f.
  * ComplexField.apply(func, out): out = func(k, v) with k the list of the
    three wavenumber arrays, broadcastable to the (n0, n1, n2//2+1) half
    spectrum.  k_d for index m is 2*pi/L_d * m for m < n_d/2 and
    2*pi/L_d * (m - n_d) for m >= n_d/2 (pmesh's circular frequency wrapped to
    [-pi, pi), so the Nyquist index carries -pi*n/L), on every axis including
    the half axis.  k.normp(p=2, zeromode=1) is sum_d |k_d|^2 with the k = 0
    entry replaced by 1.
  * csum(): the sum over the whole field (one rank: no reduction);
    cnorm(): the sum of squares.

The Nyquist convention of the gradient (-i k_d at the Nyquist index) is the
one place where pmesh's exact arithmetic is not restated: how a c2r treats
the non-Hermitian content an odd operator leaves there depends on the FFT
library.  The fixtures are made on meshes whose spacing keeps the filtered
Nyquist modes below exp(-sigma^2 k_N^2) ~ 1e-11 of the signal, so the choice
does not show at any tolerance the tests use.
"""
import numpy as np

try:
    import scipy.fft as _fft

    def _rfftn(a):
        return _fft.rfftn(a)

    def _irfftn(a, s):
        return _fft.irfftn(a, s=s, axes=(0, 1, 2))
except ImportError:  # pragma: no cover
    def _rfftn(a):
        return np.fft.rfftn(a)

    def _irfftn(a, s):
        return np.fft.irfftn(a, s=s, axes=(0, 1, 2))


class _Wavenumbers(list):
    """The k list passed to apply() transfer functions."""

    def normp(self, p=2, zeromode=None):
        out = sum(np.abs(k) ** p for k in self)
        out = np.broadcast_to(out, np.broadcast_shapes(*(k.shape for k in self))).copy()
        if zeromode is not None:
            out[0, 0, 0] = zeromode
        return out


class _Field(np.ndarray):
    """Common base: a numpy array that remembers its mesh."""

    def __array_finalize__(self, obj):
        self.pm = getattr(obj, "pm", None)

    @property
    def value(self):
        return self.view(np.ndarray)

    def csum(self):
        return np.sum(self.value)

    def cnorm(self):
        return np.sum(np.abs(self.value) ** 2)


class RealField(_Field):
    def r2c(self, out=None):
        pm = self.pm
        spec = _rfftn(self.value) / float(np.prod(pm.Nmesh))
        if out is None or out is Ellipsis:
            out = pm.create("complex")
        out.value[...] = spec
        return out

    def readout(self, pos, layout=None, resampler=None):
        return self.pm._readout(self.value, pos)


class ComplexField(_Field):
    def c2r(self, out=None):
        pm = self.pm
        real = _irfftn(self.value * float(np.prod(pm.Nmesh)), tuple(pm.Nmesh))
        if out is None or out is Ellipsis:
            out = pm.create("real")
        out.value[...] = real
        return out

    def apply(self, func, kind="wavenumber", out=None):
        if kind != "wavenumber":
            raise NotImplementedError(kind)
        res = func(self.pm.k, self.value.copy())
        if out is None:
            out = self.pm.create("complex")
        elif out is Ellipsis:
            out = self
        out.value[...] = res
        return out


class ParticleMesh:
    def __init__(self, Nmesh, BoxSize=1.0, dtype="f8", comm=None, resampler="cic"):
        n = np.asarray(Nmesh, dtype=np.int64).reshape(-1)
        if n.size == 1:
            n = np.repeat(n, 3)
        self.Nmesh = n
        box = np.asarray(BoxSize, dtype=np.float64).reshape(-1)
        if box.size == 1:
            box = np.repeat(box, 3)
        self.BoxSize = box.copy()
        self.dtype = np.dtype(dtype)
        self.comm = comm
        ks = []
        for d in range(3):
            m = np.arange(n[d], dtype=np.float64)
            m[m >= n[d] / 2] -= n[d]
            if d == 2:
                m = m[: n[d] // 2 + 1]
            shape = [1, 1, 1]
            shape[d] = m.size
            ks.append((2 * np.pi / box[d] * m).reshape(shape))
        self.k = _Wavenumbers(ks)

    def create(self, type="real", value=None):
        if type == "real":
            shape = tuple(int(x) for x in self.Nmesh)
            arr = np.zeros(shape, dtype=self.dtype).view(RealField)
        elif type == "complex":
            shape = (int(self.Nmesh[0]), int(self.Nmesh[1]), int(self.Nmesh[2]) // 2 + 1)
            cdt = np.complex64 if self.dtype == np.float32 else np.complex128
            arr = np.zeros(shape, dtype=cdt).view(ComplexField)
        else:
            raise ValueError(type)
        arr.pm = self
        if value is not None:
            arr.value[...] = value
        return arr

    def decompose(self, pos, smoothing=None):
        return None

    def _corners(self, pos):
        s = np.asarray(pos, dtype=np.float64) * (self.Nmesh / self.BoxSize)[None, :]
        i0 = np.floor(s).astype(np.int64)
        f = s - i0
        for dx in (0, 1):
            wx = f[:, 0] if dx else 1.0 - f[:, 0]
            ix = (i0[:, 0] + dx) % self.Nmesh[0]
            for dy in (0, 1):
                wy = f[:, 1] if dy else 1.0 - f[:, 1]
                iy = (i0[:, 1] + dy) % self.Nmesh[1]
                for dz in (0, 1):
                    wz = f[:, 2] if dz else 1.0 - f[:, 2]
                    iz = (i0[:, 2] + dz) % self.Nmesh[2]
                    yield (ix * self.Nmesh[1] + iy) * self.Nmesh[2] + iz, wx * wy * wz

    def paint(self, pos, mass=1.0, layout=None, out=None, hold=False, resampler=None):
        pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
        w = np.broadcast_to(np.asarray(mass, dtype=np.float64), (len(pos),))
        M = int(np.prod(self.Nmesh))
        acc = np.zeros(M, dtype=np.float64)
        for flat, wt in self._corners(pos):
            acc += np.bincount(flat, weights=w * wt, minlength=M)
        if out is None:
            out = self.create("real")
        if hold:
            out.value[...] += acc.reshape(out.shape)
        else:
            out.value[...] = acc.reshape(out.shape)
        return out

    def _readout(self, grid, pos):
        pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
        flatgrid = np.asarray(grid).reshape(-1)
        out = np.zeros(len(pos), dtype=np.float64)
        for flat, wt in self._corners(pos):
            out += wt * flatgrid[flat]
        return out.astype(grid.dtype, copy=False)
