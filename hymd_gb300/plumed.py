"""PLUMED bias coupling -- drop-in for hymd/plumed.py:11-235 (PlumedBias).

The bias is a host library: every outer step the positions go to PLUMED,
which returns bias forces and the bias energy.  PlumedBias speaks PLUMED's
`cmd` protocol exactly as the reference does (same commands, order and
units); `kernel` may be any object with a `cmd(name, value=None)` method
(default: py-plumed's `plumed.Plumed()`).  The device MD loop
(RespaMD.set_bias) copies positions and the current forces to the host,
calls prepare/calc, and adds the returned bias force to the slow forces of
the outer kicks, as hymd/main.py:808-812 and 1097-1154 do.
"""
import logging
import os

import numpy as np

log = logging.getLogger("hymd_gb300")


def _host(x, dtype=np.double):
    try:
        import torch
        if isinstance(x, torch.Tensor):
            x = x.detach().cpu().numpy()
    except ImportError:  # pragma: no cover
        pass
    return np.asarray(x, dtype=dtype)


def _host_raw(x):
    """x on the host as a numpy array in its own dtype (no conversion)."""
    try:
        import torch
        if isinstance(x, torch.Tensor):
            return x.detach().cpu().numpy()
    except ImportError:  # pragma: no cover
        pass
    return np.asarray(x)


class PlumedBias:
    """PLUMED handler (hymd/plumed.py:11-235): construct once, then per step
    prepare() (positions, current forces; returns whether PLUMED needs the
    potential energy) and calc() (returns the bias forces and energy)."""

    def __init__(self, config, plumeddat, logfile, intracomm=None, intercomm=None, verbose=1,
                 kernel=None):
        self.verbose = verbose
        self.intracomm = intracomm
        self.intercomm = intercomm
        self.ready = False
        self.plumed_bias = np.zeros(1, np.double)
        self.plumed_version = np.zeros(1, dtype=np.intc)
        self.plumed_forces = None
        self.positions = None
        self.charges = None
        if kernel is None:
            try:
                import plumed
            except ImportError:
                msg = "You are trying to use PLUMED but HyMD could not import py-plumed."
                log.error(msg)
                raise ImportError(msg)
            k = os.environ.get("PLUMED_KERNEL")
            log.info("Using PLUMED_KERNEL=%s" % k if k else
                     "The PLUMED_KERNEL environment variable is not set.")
            try:
                kernel = plumed.Plumed()
            except Exception as e:
                msg = ("HyMD was not able to create a PLUMED object. "
                       "Maybe there is a problem with your PLUMED_KERNEL?")
                log.error(msg)
                raise RuntimeError(msg) from e
        self.plumed_obj = kernel
        kernel.cmd("getApiVersion", self.plumed_version)
        if self.plumed_version[0] <= 3:
            msg = "HyMD requires a PLUMED API > 3. Use a newer PLUMED kernel."
            log.error(msg)
            raise AssertionError(msg)
        kernel.cmd("setMDEngine", "HyMD")
        if intercomm is not None:  # multi-replica runs are not wired on one GPU
            raise NotImplementedError("PLUMED replica exchange (intercomm)")
        log.info("Attempting to read PLUMED input from %s", plumeddat)
        kernel.cmd("setPlumedDat", plumeddat)
        kernel.cmd("setLogFile", logfile)
        kernel.cmd("setTimestep", config.respa_inner * config.time_step)
        kernel.cmd("setNatoms", config.n_particles)
        kernel.cmd("setKbT", config.gas_constant * config.target_temperature)
        kernel.cmd("setNoVirial")
        kernel.cmd("init")
        log.info("Successfully read PLUMED input. PLUMED output file is %s", logfile)

    def finalize(self):
        fin = getattr(self.plumed_obj, "finalize", None)
        if fin is not None:
            fin()

    def __enter__(self):
        return self

    def __exit__(self, exc_type, exc_value, traceback):
        ex = getattr(self.plumed_obj, "__exit__", None)
        if ex is not None:
            ex(exc_type, exc_value, traceback)
        else:
            self.finalize()

    @property
    def api_version(self):
        return self.plumed_version[0]

    def prepare(self, step, forces, positions, indices, config, charges):
        """Hand PLUMED the step's positions, forces (copied; PLUMED adds the
        bias into the copy), charges, masses and box (hymd/plumed.py:176-213);
        returns True if PLUMED asks for the potential energy."""
        if self.verbose > 1:
            log.info("Setting PLUMED pointers for step %d", step)
        # float64 copies, as the reference's astype(np.double) makes them
        # (PLUMED adds the bias into the force array), held in buffers that
        # persist between steps: fresh arrays of this size fault their pages
        # in every step
        f_in = _host_raw(forces)
        self.plumed_forces = self._copy("_plumed_f", f_in)
        self.charges = self._copy("_charges", _host_raw(charges))
        self.positions = self._copy("_positions", _host_raw(positions))
        idx = np.ascontiguousarray(_host(indices, np.intc))
        needs_energy = np.zeros(1, np.intc)
        masses = getattr(self, "_masses", None)
        if masses is None or masses.shape[0] != idx.shape[0] or masses[0] != config.mass:
            masses = self._masses = np.full(idx.shape[0], config.mass, dtype=np.double)
        box = np.diag(_host(config.box_size)).astype(np.double)
        k = self.plumed_obj
        k.cmd("setAtomsNlocal", idx.shape[0])
        k.cmd("setAtomsGatindex", idx)
        k.cmd("setStep", step)
        k.cmd("setForces", self.plumed_forces)
        k.cmd("setPositions", self.positions)
        k.cmd("setCharges", self.charges)
        k.cmd("setMasses", masses)
        k.cmd("setBox", box)
        k.cmd("prepareCalc")
        k.cmd("isEnergyNeeded", needs_energy)
        self._shape = tuple(f_in.shape)
        self.ready = True
        return bool(needs_energy[0] != 0)

    def _copy(self, name, x):
        """x flattened into the float64 buffer `name` (allocated on first use
        or when the size changes)."""
        buf = getattr(self, name, None)
        if buf is None or buf.shape[0] != x.size:
            buf = np.empty(x.size, dtype=np.double)
            setattr(self, name, buf)
        np.copyto(buf, x.reshape(-1))
        return buf

    def calc(self, forces, poteng):
        """Run PLUMED on the prepared step; returns (bias forces (N, 3), bias
        energy): the forces PLUMED returned minus the forces it was given
        (hymd/plumed.py:215-235)."""
        if not self.ready:
            msg = "Trying to calculate PLUMED biased forces without first calling prepare method."
            log.error(msg)
            raise RuntimeError(msg)
        if self.verbose > 1:
            log.info("Calculating PLUMED forces")
        k = self.plumed_obj
        k.cmd("setEnergy", poteng)
        k.cmd("performCalc")
        k.cmd("getBias", self.plumed_bias)
        # min propagates NaN: NaN exactly when an element is (no mask array)
        if self.plumed_forces.size and np.isnan(np.min(self.plumed_forces)):
            msg = ("Forces returned by PLUMED are not valid. It means there's a NaN in the "
                   "computed forces, and your input should be checked. ")
            log.error(msg)
            raise RuntimeError(msg)
        # the forces given to calc (float32 inputs widen exactly to float64)
        bias_forces = (self.plumed_forces - _host_raw(forces).reshape(-1)).reshape(self._shape)
        if self.verbose > 1:
            log.info("Done calculating PLUMED forces")
        self.ready = False
        return bias_forces, float(self.plumed_bias[0])
