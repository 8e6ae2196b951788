"""H5MD output and input distribution against the reference's own
hymd/file_io.py (tests/golden/io_ref.npz, made by tests/golden/make_io_ref.py,
which ran the reference's OutDataset / store_static / store_data into an
in-memory H5 tree and its distribute_input over several rank counts).

The same inputs through hymd_gb300.file_io must give the same tree: every
group, dataset and attribute path, shape, dtype and value, except the
author name, the creator version and the config dump, which name the
writing program and user.  In the manner of the reference's
test/test_file_io.py, with the in-memory tree standing in for an h5py file.
"""
import os

import numpy as np
import pytest

from hymd_gb300 import file_io as fio

FIX = np.load(os.path.join(os.path.dirname(__file__), "golden", "io_ref.npz"))
SKIP = {"/h5md/author@name", "/h5md/creator@version", "/parameters@config.toml"}


def _config():
    from hymd_gb300.config import Config
    names, types = FIX["inputs/names"], FIX["inputs/types"]
    T = int(types.max()) + 1
    tmap = {t: names[types == t][0].decode() for t in range(T)}
    n_steps, n_print, mass, dt = FIX["inputs/scalars"]
    return Config(n_steps=int(n_steps), n_print=int(n_print), time_step=float(dt),
                  mesh_size=[5, 5, 5], sigma=0.5, kappa=0.05,
                  box_size=np.array([10.0, 10.0, 10.0]), n_particles=len(names), mass=mass,
                  n_types=T, type_to_name_map=tmap, unique_names=sorted(tmap.values()))


def _write(tmp_path):
    cfg = _config()
    out = fio.OutDataset(str(tmp_path), cfg, backend="memory")
    idx = FIX["inputs/indices"]
    fio.store_static(out, list(range(len(idx))), FIX["inputs/names"], FIX["inputs/types"], idx,
                     cfg, FIX["inputs/bond_from"], FIX["inputs/bond_to"],
                     molecules=FIX["inputs/molecules"], velocity_out=True, force_out=True,
                     charges=FIX["inputs/charges"], plumed_out=True)
    perm = FIX["frames/perm"]
    box = np.array([10.0, 10.0, 10.0])
    for frame, step in enumerate(FIX["frames/steps"]):
        g = lambda k: FIX[f"frames/{frame}/{k}"]  # noqa: E731
        sc = g("sc")
        cfg.thermostat_work = float(sc[8])
        fio.store_data(out, int(step), frame, idx[perm], g("pos")[perm], g("vel")[perm],
                       g("frc")[perm], box * (1 + 0.01 * frame), abs(sc[0]), g("pressure"),
                       abs(sc[1]), sc[2], sc[3], sc[4], sc[5], sc[6], sc[7], 0.3, cfg,
                       velocity_out=True, force_out=True, charge_out=True, plumed_out=True)
    return out


def test_output_tree_matches_reference(tmp_path):
    out = _write(tmp_path)
    got = out.file.to_dict()
    want = {k[5:]: FIX[k] for k in FIX.files if k.startswith("tree/")}
    assert set(got) == set(want)
    for k, v in want.items():
        if k in SKIP:
            continue
        g = np.asarray(got[k])
        assert g.shape == v.shape, k
        assert g.dtype == v.dtype or (g.dtype.kind == v.dtype.kind == "S"), (k, g.dtype, v.dtype)
        if v.dtype.kind == "f" and k.split("/")[2:3] in (["total_momentum"],
                                                         ["angular_momentum"], ["torque"]):
            # sums over particles: the reference adds float32 arrays in float32,
            # this code in float64
            np.testing.assert_allclose(g, v, rtol=0, atol=1e-5 * np.abs(v).max(), err_msg=k)
        elif v.dtype.kind == "f":
            np.testing.assert_allclose(g, v, rtol=1e-6, atol=0, err_msg=k)
        else:
            assert np.array_equal(g, v), k
    # the groups of the reference's own test_store_static
    f = out.file
    assert all(k in f.keys() for k in ["connectivity", "h5md", "observables", "parameters",
                                       "particles"])
    assert all(k in f["particles/all"] for k in ["box", "mass", "position", "species"])
    out.close_file()
    assert not out.is_open()
    saved = np.load(os.path.join(str(tmp_path), "sim.H5.npz"))
    assert np.array_equal(saved["/particles/all/position/value"],
                          got["/particles/all/position/value"])


def test_store_data_scalars(tmp_path):
    """The reference's test_store_data checks, on the first frame."""
    out = _write(tmp_path)
    sc = FIX["frames/0/sc"]
    pot = sc[2] + sc[3] + sc[4] + sc[5] + sc[6]
    assert out.potential_energy[0] == pytest.approx(pot, rel=1e-6)
    assert out.kinetc_energy[0] == pytest.approx(abs(sc[1]), rel=1e-6)
    assert out.total_energy[0] == pytest.approx(pot + abs(sc[1]), rel=1e-6)
    assert out.field_q_energy[0] == pytest.approx(sc[6], rel=1e-6)
    assert out.plumed_bias[0] == pytest.approx(sc[7], rel=1e-6)
    for d in (out.positions_step, out.total_energy_step, out.thermostat_work_step):
        assert d[0] == 0


@pytest.mark.parametrize("size", [1, 2, 3, 4, 7])
def test_distribute_input_matches_reference(size):
    n = 10000
    idx = np.arange(n)
    mol = np.zeros(n, np.int64)
    mol[400:450] = 1
    mol[450:] = np.arange(2, 9552)
    covered = []
    for rank in range(size):
        r1, f1 = fio.distribute_input({"indices": idx}, rank, size, None)
        r2, f2 = fio.distribute_input({"indices": idx, "molecules": mol}, rank, size, n,
                                      max_molecule_size=1000)
        assert not f1 and f2
        assert [r1[0], r1[-1] + 1] == list(FIX[f"dist/{size}/{rank}/none"])
        assert [r2[0], r2[-1] + 1] == list(FIX[f"dist/{size}/{rank}/mol"])
        covered += r2
    assert covered == list(range(n))  # no gaps, no overlaps, molecules whole


def test_frame_count():
    # hymd/file_io.py:204-211 on a few (n_steps, n_print) pairs
    assert fio.n_output_frames(10, 3) == 4
    assert fio.n_output_frames(100, 1) == 101
    assert fio.n_output_frames(100, 10) == 11
    assert fio.n_output_frames(1, 1) == 2


def test_store_data_contiguous_rows_match_sorted_write(tmp_path):
    """Rows that already hold the consecutive ascending global indices are
    written as one slice; the frames equal those of the reference's
    sort-then-scatter write of the same rows in another order, and the
    momentum sums agree to summation order."""
    cfg = _config()
    idx = FIX["inputs/indices"]
    order = np.argsort(idx)
    box = np.array([10.0, 10.0, 10.0])
    outs = []
    for k, (rows, ix) in enumerate(((order, idx[order]), (FIX["frames/perm"], None))):
        out = fio.OutDataset(str(tmp_path / str(k)), cfg, backend="memory")
        fio.store_static(out, list(range(len(idx))), FIX["inputs/names"], FIX["inputs/types"],
                         idx, cfg, FIX["inputs/bond_from"], FIX["inputs/bond_to"],
                         molecules=FIX["inputs/molecules"], velocity_out=True, force_out=True)
        ix = idx[rows] if ix is None else ix
        for frame, step in enumerate(FIX["frames/steps"]):
            g = lambda key: FIX[f"frames/{frame}/{key}"][rows]  # noqa: E731
            fio.store_data(out, int(step), frame, ix, g("pos"), g("vel"), g("frc"), box, 300.0,
                           0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.3, cfg,
                           velocity_out=True, force_out=True)
        outs.append(out)
    assert np.array_equal(idx[order], np.arange(idx[order][0], idx[order][0] + len(idx)))
    a, b = outs
    for name in ("positions", "velocities", "forces"):
        assert np.array_equal(getattr(a, name)[:], getattr(b, name)[:]), name
    for name in ("total_momentum", "angular_momentum", "torque"):
        np.testing.assert_allclose(getattr(a, name)[:], getattr(b, name)[:], rtol=1e-12,
                                   atol=1e-12, err_msg=name)


def test_store_data_concurrent_threads(tmp_path):
    """store_data from two threads at once (trajectory writer threads of two
    runs): each tree gets its own frames and momentum sums, the same as
    written one after the other."""
    import threading
    cfg = _config()
    idx = FIX["inputs/indices"]
    order = np.argsort(idx)
    box = np.array([10.0, 10.0, 10.0])
    steps = FIX["frames/steps"]
    # the archive is read here, once: an npz file is not safe to read from
    # two threads
    data = {(f, k): FIX[f"frames/{f}/{k}"][order] for f in range(len(steps))
            for k in ("pos", "vel", "frc")}

    def write(out, scale, reps):
        for _ in range(reps):
            for frame, step in enumerate(steps):
                g = lambda key: scale * data[(frame, key)]  # noqa: E731
                fio.store_data(out, int(step), frame, idx[order], g("pos"), g("vel"), g("frc"),
                               box, 300.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.3, cfg,
                               velocity_out=True, force_out=True)

    def new_out(tag):
        out = fio.OutDataset(str(tmp_path / tag), cfg, backend="memory")
        fio.store_static(out, list(range(len(idx))), FIX["inputs/names"], FIX["inputs/types"],
                         idx, cfg, FIX["inputs/bond_from"], FIX["inputs/bond_to"],
                         molecules=FIX["inputs/molecules"], velocity_out=True, force_out=True)
        return out

    seq = [new_out("s1"), new_out("s2")]
    write(seq[0], 1.0, 1)
    write(seq[1], 2.0, 1)
    par = [new_out("p1"), new_out("p2")]
    th = [threading.Thread(target=write, args=(par[k], 1.0 + k, 50)) for k in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for a, b in zip(seq, par):
        for name in ("positions", "total_momentum", "angular_momentum", "torque"):
            assert np.array_equal(getattr(a, name)[:], getattr(b, name)[:]), name
