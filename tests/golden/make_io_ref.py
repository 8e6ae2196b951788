"""Generate tests/golden/io_ref.npz from the reference's own hymd/file_io.py.

    python tests/golden/make_io_ref.py <path-to-HyMD-checkout>
    (or set HYMD_REFERENCE)

h5py is not installed here, so the stub h5py module of make_golden.py gets a
`File` that returns an in-memory H5 tree (hymd_gb300.file_io.H5Tree); the
reference's unmodified OutDataset, store_static and store_data then write
their H5MD layout into it.  Inputs: the molecules_with_solvent system of the
reference's test/conftest.py, its bonds from the reference's prepare_bonds,
and frames of seeded synthetic data.  Also records distribute_input's rank
ranges for several communicator sizes, with and without molecules.

Keys: tree/<dataset path> and tree/<path>@<attribute> (the output file),
inputs/*, frames/* (what store_data was given), dist/<size>/<rank>/<mol>,
and plumed/* (the reference's PLUMED test input and its golden outputs:
refforces.txt, refDIST, reftestdump.xyz and the asserted bias).
"""
import os
import sys
import tempfile
import types as _types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

import make_golden as mg  # noqa: E402
from hymd_gb300.file_io import H5Tree  # noqa: E402

N_STEPS, N_PRINT = 10, 3


def main(ref):
    import warnings
    warnings.filterwarnings("ignore", category=SyntaxWarning)
    mg._install_stubs()
    sys.modules["h5py"].File = lambda *a, **k: H5Tree()
    sys.modules["h5py"].Dataset = object
    pkg = _types.ModuleType("hymd")
    pkg.__path__ = [os.path.join(ref, "hymd")]
    sys.modules["hymd"] = pkg
    R = {}
    for name in ("version", "logger", "force", "barostat", "input_parser", "file_io"):
        R[name] = mg._load("hymd." + name, os.path.join(ref, "hymd", name + ".py"), "hymd")
    R["force"].Logger = R["logger"].Logger
    import logging
    R["force"].logging = logging
    conft = mg._load("ref_conftest", os.path.join(ref, "test", "conftest.py"))
    fio = R["file_io"]
    ip = R["input_parser"]
    indices, positions, molecules, velocities, bonds, names, types = conft.molecules_with_solvent()
    box = np.array([10.0, 10.0, 10.0])
    Tp = R["barostat"].Target_pressure
    config = ip.Config(n_steps=N_STEPS, n_print=N_PRINT, time_step=0.03, box_size=box,
                       mesh_size=[5, 5, 5], sigma=0.5, kappa=0.05, n_particles=len(indices),
                       mass=72.0, target_pressure=Tp(P_L=None, P_N=None))
    B = R["force"].Bond
    config.bonds = [B("A", "A", 0.27, 10000.0), B("A", "B", 0.27, 10000.0),
                    B("A", "C", 0.27, 10000.0), B("B", "B", 0.27, 10000.0),
                    B("B", "C", 0.27, 10000.0)]
    config = ip._setup_type_to_name_map(config, names, types)
    in_file = {"molecules": molecules, "indices": indices}
    rank_range, _ = fio.distribute_input(in_file, 0, 1, config.n_particles, 6)
    packed = R["force"].prepare_bonds(molecules[rank_range], names[rank_range],
                                      bonds[rank_range], indices[rank_range], config)
    rng = np.random.default_rng(3)
    charges = rng.choice([-1.0, 0.0, 1.0], len(indices)).astype(np.float32)
    out = fio.OutDataset(tempfile.gettempdir(), config)
    fio.store_static(out, rank_range, names, types, indices, config, packed[0], packed[1],
                     molecules=molecules, velocity_out=True, force_out=True, charges=charges,
                     plumed_out=True)
    res = {"inputs/indices": indices, "inputs/positions": positions,
           "inputs/molecules": molecules, "inputs/velocities": velocities, "inputs/bonds": bonds,
           "inputs/names": names, "inputs/types": types, "inputs/charges": charges,
           "inputs/bond_from": np.asarray(packed[0]), "inputs/bond_to": np.asarray(packed[1]),
           "inputs/scalars": np.array([N_STEPS, N_PRINT, 72.0, 0.03])}
    perm = rng.permutation(len(indices))  # rows arrive in a rank's own order
    frames = []
    for frame, step in enumerate(range(0, N_STEPS, N_PRINT)):
        pos = rng.uniform(0, 10, positions.shape).astype(np.float32)
        vel = rng.normal(0, 0.3, positions.shape).astype(np.float32)
        frc = rng.normal(0, 30.0, positions.shape).astype(np.float32)
        sc = rng.normal(0, 100.0, 9)
        pressure = rng.normal(0, 10.0, 18)
        config.thermostat_work = float(sc[8])
        fio.store_data(out, step, frame, indices[perm], pos[perm], vel[perm], frc[perm],
                       box * (1 + 0.01 * frame), abs(sc[0]), pressure, abs(sc[1]), sc[2], sc[3],
                       sc[4], sc[5], sc[6], sc[7], 0.3, config, velocity_out=True,
                       force_out=True, charge_out=True, plumed_out=True)
        for k, v in (("pos", pos), ("vel", vel), ("frc", frc), ("sc", sc),
                     ("pressure", pressure)):
            res[f"frames/{frame}/{k}"] = v
        frames.append(step)
    res["frames/steps"] = np.array(frames)
    res["frames/perm"] = perm
    for k, v in out.file.to_dict().items():
        res["tree/" + k] = v
    # distribute_input over communicator sizes
    n = 10000
    idx = np.arange(n)
    mol = np.zeros(n, np.int64)
    mol[400:450] = 1
    mol[450:] = np.arange(2, 9552)
    for size in (1, 2, 3, 4, 7):
        for rank in range(size):
            r1, _ = fio.distribute_input({"indices": idx}, rank, size, None)
            r2, _ = fio.distribute_input({"indices": idx, "molecules": mol}, rank, size, n,
                                         max_molecule_size=1000)
            res[f"dist/{size}/{rank}/none"] = np.array([r1[0], r1[-1] + 1])
            res[f"dist/{size}/{rank}/mol"] = np.array([r2[0], r2[-1] + 1])
    # the reference's PLUMED test goldens (test/test_plumed.py with
    # test/refforces.txt, refDIST, reftestdump.xyz), read as text
    import re
    tdir = os.path.join(ref, "test")
    res["plumed/ref_forces"] = np.loadtxt(os.path.join(tdir, "refforces.txt"))
    res["plumed/ref_dist"] = np.loadtxt(os.path.join(tdir, "refDIST"))
    dump = open(os.path.join(tdir, "reftestdump.xyz")).read().splitlines()
    res["plumed/ref_dump_box"] = np.array([float(x) for x in dump[1].split()])
    res["plumed/ref_dump"] = np.array([[float(x) for x in ln.split()[1:]] for ln in dump[2:]])
    src = open(os.path.join(tdir, "test_plumed.py")).read()
    res["plumed/ref_bias"] = np.array(float(
        re.search(r"plumed_bias == pytest.approx\(([0-9.eE+-]+)", src).group(1)))
    res["plumed/input"] = np.array(re.search(r'plumed_str = """(.*?)"""', src, re.S).group(1))
    path = os.path.join(HERE, "io_ref.npz")
    np.savez_compressed(path, **res)
    print("wrote", path, os.path.getsize(path), "bytes,", len(res), "arrays")


if __name__ == "__main__":
    main(mg.reference_root())
