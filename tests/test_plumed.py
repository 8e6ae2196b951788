"""PlumedBias (hymd_gb300/plumed.py) against the reference's own PLUMED test
(test/test_plumed.py:11-120): the same input (a DISTANCE between atoms 1 and
4 with a RESTRAINT at 2 nm, KAPPA 200), the molecules_with_solvent system,
and its golden outputs -- the bias forces (refforces.txt), the bias
635.5621691482, the printed distance (refDIST) and the dumped atoms
(reftestdump.xyz) -- with tests/plumed_fake.py standing in for the PLUMED
library, which is not installed here.
"""
import builtins
import os

import numpy as np
import pytest

from plumed_fake import FakePlumed

FIX = np.load(os.path.join(os.path.dirname(__file__), "golden", "io_ref.npz"))


def _config():
    from hymd_gb300.config import Config
    return Config(n_steps=1, time_step=0.03, box_size=np.array([10.0, 10.0, 10.0]),
                  mesh_size=[5, 5, 5], sigma=0.5, kappa=0.05,
                  n_particles=len(FIX["inputs/indices"]), target_temperature=300.0, mass=72.0)


def test_plumed_bias_matches_reference_goldens(tmp_path):
    from hymd_gb300.plumed import PlumedBias
    text = str(FIX["plumed/input"]).format(os.path.join(tmp_path, "testdump.xyz"),
                                           os.path.join(tmp_path, "DIST"))
    dat = os.path.join(tmp_path, "plumed.dat")
    with open(dat, "w") as f:
        f.write(text)
    cfg = _config()
    kernel = FakePlumed()
    bias = PlumedBias(cfg, dat, os.path.join(tmp_path, "plumed.out"), verbose=2, kernel=kernel)
    assert bias.api_version > 3
    pos = FIX["inputs/positions"]
    idx = FIX["inputs/indices"].astype(np.intc)
    forces = np.zeros_like(pos)
    charges = np.zeros_like(idx, dtype=np.double)
    assert bias.prepare(0, forces, pos, idx, cfg, charges) is False
    f_bias, e_bias = bias.calc(forces, 0.0)
    ref = FIX["plumed/ref_forces"]
    assert f_bias[: len(ref)] == pytest.approx(ref, abs=1e-8)
    assert np.all(f_bias[len(ref):] == 0.0)
    assert e_bias == pytest.approx(float(FIX["plumed/ref_bias"]), abs=1e-8)
    bias.finalize()
    dist = np.loadtxt(os.path.join(tmp_path, "DIST"))
    assert np.allclose(dist, FIX["plumed/ref_dist"], atol=1e-6)
    lines = open(os.path.join(tmp_path, "testdump.xyz")).read().splitlines()
    assert int(lines[0]) == len(FIX["plumed/ref_dump"])
    assert np.allclose([float(x) for x in lines[1].split()], FIX["plumed/ref_dump_box"])
    dump = np.array([[float(x) for x in ln.split()[1:]] for ln in lines[2:]])
    # the reference's dump comes from its two-rank run, whose atom order in
    # the file follows that run's decomposition: the same 45 positions in
    # another order, so compare them as a set of rows
    key = lambda a: sorted(map(tuple, np.round(a, 5)))  # noqa: E731
    assert key(dump) == key(FIX["plumed/ref_dump"])
    # the reference's command sequence of a step
    seq = kernel.calls
    i = seq.index("setAtomsNlocal")
    assert seq[i:i + 11] == ["setAtomsNlocal", "setAtomsGatindex", "setStep", "setForces",
                             "setPositions", "setCharges", "setMasses", "setBox", "prepareCalc",
                             "isEnergyNeeded", "setEnergy"]
    with pytest.raises(RuntimeError, match="without first calling prepare method"):
        bias.calc(forces, 0.0)


def test_bias_adds_to_given_forces(tmp_path):
    """calc() returns only the bias: the forces handed to prepare() come back
    unchanged underneath it."""
    from hymd_gb300.plumed import PlumedBias
    dat = os.path.join(tmp_path, "plumed.dat")
    with open(dat, "w") as f:
        f.write("d: DISTANCE ATOMS=2,7\nRESTRAINT ARG=d KAPPA=50.0 AT=0.5\n")
    cfg = _config()
    bias = PlumedBias(cfg, dat, os.path.join(tmp_path, "log"), kernel=FakePlumed())
    pos = FIX["inputs/positions"]
    idx = FIX["inputs/indices"].astype(np.intc)
    base = np.random.default_rng(1).normal(0, 10, pos.shape)
    bias.prepare(3, base, pos, idx, cfg, np.zeros(len(idx)))
    f1, e1 = bias.calc(base, 0.0)
    bias.prepare(3, np.zeros_like(pos), pos, idx, cfg, np.zeros(len(idx)))
    f2, e2 = bias.calc(np.zeros_like(pos), 0.0)
    assert np.allclose(f1, f2, atol=1e-9) and e1 == pytest.approx(e2)
    assert np.count_nonzero(np.abs(f1).sum(1)) == 2
    assert np.allclose(f1.sum(0), 0.0, atol=1e-9)  # a pair force: no net force


def test_unavailable_plumed(monkeypatch):
    from hymd_gb300.plumed import PlumedBias
    real = builtins.__import__

    def no_plumed(name, *a, **k):
        if name == "plumed":
            raise ImportError()
        return real(name, *a, **k)

    monkeypatch.setattr(builtins, "__import__", no_plumed)
    with pytest.raises(ImportError, match="could not import py-plumed"):
        PlumedBias(_config(), "test.in", "test.out")
