"""H5MD trajectory and observable output, and input distribution -- drop-in
for hymd/file_io.py (OutDataset :12-88, setup_time_dependent_element
:91-119, store_static :122-525, store_data :527-779, distribute_input
:781-874).

The output layout is the reference's H5MD tree (group, dataset and attribute
names, shapes, dtypes, units, frame count), written through h5py when it is
importable.  Without h5py the same tree is built in memory (`H5Tree`) and
saved as a compressed .npz on close (one array per dataset path, attributes
as "<path>@<name>"), so the output exists on machines without HDF5; a caller
can also pass any object with h5py's group/dataset interface as `file`.

One process owns the whole system here, so the MPI pieces reduce to one
rank: `comm` is accepted and ignored, and parallel HDF5 (mpio) is not used.
`TrajectoryRecorder` (hymd_gb300.trajectory) feeds store_data from the
device without stalling the step.
"""
import getpass
import logging
import os
import threading

import numpy as np

log = logging.getLogger("hymd_gb300")

__version__ = "0.2"


# ---------------------------------------------------------------- in-memory
class _Attrs(dict):
    pass


class Dataset:
    """A fixed-shape numpy array with h5py-like indexing and attributes."""

    def __init__(self, name, shape, dtype):
        self.name = name
        self.value = np.zeros(shape, dtype=np.dtype(dtype))
        # commit the pages now (zeros are mapped lazily), so that the frames
        # written during the run do not fault them in one by one
        if self.value.dtype.kind in "fiu":
            self.value.fill(0)
        self.attrs = _Attrs()

    @property
    def shape(self):
        return self.value.shape

    @property
    def dtype(self):
        return self.value.dtype

    def __getitem__(self, key):
        return self.value[key]

    def __setitem__(self, key, val):
        self.value[key] = val

    def __len__(self):
        return len(self.value)


class Group:
    """A node of the tree: child groups and datasets by name, attributes."""

    def __init__(self, name):
        self.name = name
        self.attrs = _Attrs()
        self._children = {}

    def _path(self, child):
        return ("" if self.name == "/" else self.name) + "/" + child

    def _walk(self, path, create):
        node = self
        parts = [p for p in path.split("/") if p]
        if path.startswith("/"):
            node = self._root()
        for p in parts[:-1]:
            if p not in node._children:
                if not create:
                    raise KeyError(path)
                node._children[p] = Group(node._path(p))
                node._children[p]._parent = node
            node = node._children[p]
        return node, parts[-1]

    def _root(self):
        node = self
        while getattr(node, "_parent", None) is not None:
            node = node._parent
        return node

    def create_group(self, name):
        node, leaf = self._walk(name, True)
        if leaf in node._children:
            raise ValueError(f"{name}: exists")
        g = Group(node._path(leaf))
        g._parent = node
        node._children[leaf] = g
        return g

    def create_dataset(self, name, shape=None, dtype="float32", data=None):
        node, leaf = self._walk(name, True)
        if leaf in node._children:
            raise ValueError(f"{name}: exists")
        if data is not None:
            data = np.asarray(data)
            shape = data.shape if shape is None else shape
            dtype = data.dtype if dtype is None else dtype
        d = Dataset(node._path(leaf), tuple(np.atleast_1d(shape)) if shape is not None else (),
                    dtype)
        if data is not None:
            d.value[...] = data
        node._children[leaf] = d
        return d

    def __getitem__(self, path):
        node, leaf = self._walk(path, False)
        return node._children[leaf]

    def __contains__(self, path):
        try:
            self[path]
            return True
        except KeyError:
            return False

    def keys(self):
        return list(self._children.keys())

    def items(self):
        return list(self._children.items())


class H5Tree(Group):
    """An in-memory H5-like file; `close()` saves it to `path` (if given) as a
    compressed .npz of every dataset and attribute."""

    def __init__(self, path=None):
        super().__init__("/")
        self._parent = None
        self.path = path
        self._open = True

    def __bool__(self):
        return self._open

    def flush(self):
        pass

    def close(self):
        if self._open and self.path:
            np.savez_compressed(self.path, **self.to_dict())
        self._open = False

    def to_dict(self):
        """{dataset path: array, "<path>@<attr>": attribute value} of the tree."""
        out = {}

        def walk(node):
            for k, v in node.attrs.items():
                out[f"{node.name}@{k}"] = np.asarray(v)
            if isinstance(node, Dataset):
                out[node.name] = node.value
                return
            for child in node._children.values():
                walk(child)

        walk(self)
        return out


def _h5py():
    try:
        import h5py
        return h5py
    except ImportError:
        return None


# ------------------------------------------------------------ the dataset
class OutDataset:
    """HDF5 dataset handler for file output (hymd/file_io.py:12-88).

    backend: "h5py" (needs h5py), "memory" (an H5Tree saved to
    <dest_directory>/sim.H5.npz on close) or "auto" (h5py when importable,
    else memory).  `file` overrides both with a caller's h5py-like object."""

    def __init__(self, dest_directory, config, double_out=False, disable_mpio=False, comm=None,
                 backend="auto", file=None):
        self.disable_mpio = disable_mpio
        self.config = config
        self.float_dtype = "float64" if double_out else "float32"
        if file is not None:
            self.file = file
            return
        h5py = _h5py() if backend in ("auto", "h5py") else None
        if backend == "h5py" and h5py is None:
            raise ImportError("OutDataset(backend='h5py') needs h5py")
        name = "sim.hdf5-     0-of-     1" if disable_mpio else "sim.H5"
        if h5py is not None:
            self.file = h5py.File(os.path.join(dest_directory, name), "w")
        else:
            self.file = H5Tree(os.path.join(dest_directory, name + ".npz"))

    def is_open(self, comm=None):
        return bool(self.file)

    def close_file(self, comm=None):
        self.file.close()

    def flush(self):
        self.file.flush()


def setup_time_dependent_element(name, parent_group, n_frames, shape, dtype, units=None):
    """An H5MD time-dependent element: group `name` with datasets step
    (n_frames,) int32, time (n_frames,) float32 and value (n_frames, *shape)
    (hymd/file_io.py:91-119)."""
    group = parent_group.create_group(name)
    step = group.create_dataset("step", (n_frames,), "int32")
    time = group.create_dataset("time", (n_frames,), "float32")
    value = group.create_dataset("value", (n_frames, *shape), dtype)
    if units is not None:
        value.attrs["unit"] = units
        time.attrs["unit"] = "ps"
    return group, step, time, value


def n_output_frames(n_steps, n_print):
    """Frames allocated for a run of n_steps with output every n_print
    steps, including the frame of step 0, as hymd/file_io.py:204-211
    counts them."""
    n = n_steps // n_print
    if (n_steps - 1) % n_print != 0:
        n += 1
    if n_steps % n_print == 1:
        n += 1
    if n == n_steps:
        n += 1
    return n


def _name_to_type(config):
    m = getattr(config, "name_to_type_map", None)
    if m:
        return m
    return {v: k for k, v in config.type_to_name_map.items()}


# the per-frame observables of store_static / store_data, in the order the
# reference creates them: (attribute prefix, element name, shape, dtype, unit)
def _observables(dtype, charges, plumed_out):
    obs = [("total_energy", "total_energy", (1,), dtype, "kJ mol-1"),
           ("kinetc_energy", "kinetic_energy", (1,), dtype, "kJ mol-1"),
           ("potential_energy", "potential_energy", (1,), dtype, "kJ mol-1"),
           ("bond_energy", "bond_energy", (1,), dtype, "kJ mol-1"),
           ("angle_energy", "angle_energy", (1,), dtype, "kJ mol-1"),
           ("dihedral_energy", "dihedral_energy", (1,), dtype, "kJ mol-1"),
           ("field_energy", "field_energy", (1,), dtype, "kJ mol-1")]
    if charges is not False:
        obs.append(("field_q_energy", "field_q_energy", (1,), dtype, "kJ mol-1"))
    if plumed_out is not False:
        obs.append(("plumed_bias", "plumed_bias", (1,), dtype, "kJ mol-1"))
    obs += [("total_momentum", "total_momentum", (3,), dtype, "nm g ps-1 mol-1"),
            ("angular_momentum", "angular_momentum", (3,), dtype, "nm+2 g ps-1 mol-1"),
            ("torque", "torque", (3,), dtype, "kJ nm+2 mol-1"),
            ("temperature", "temperature", (3,), dtype, "K"),
            ("thermostat_work", "thermostat_work", (1,), "float32", "kJ mol-1"),
            ("pressure", "pressure", (18,), "float32", "Bar")]
    return obs


def store_static(h5md, rank_range, names, types, indices, config, bonds_2_atom1,
                 bonds_2_atom2, molecules=None, velocity_out=False, force_out=False,
                 charges=False, dielectrics=False, plumed_out=False, comm=None):
    """The time-independent part of the output and the time-dependent
    elements, sized for the run's frame count (hymd/file_io.py:122-525)."""
    dtype = h5md.float_dtype
    f = h5md.file
    h5md.h5md_group = f.create_group("/h5md")
    h5md.observables = f.create_group("/observables")
    h5md.connectivity = f.create_group("/connectivity")
    h5md.parameters = f.create_group("/parameters")
    h5md.h5md_group.attrs["version"] = np.array([1, 1], dtype=int)
    h5md.h5md_group.create_group("author").attrs["name"] = np.bytes_(getpass.getuser())
    creator = h5md.h5md_group.create_group("creator")
    creator.attrs["name"] = np.bytes_("Hylleraas MD")
    creator.attrs["version"] = np.bytes_(f"hymd_gb300 {__version__}")
    h5md.particles_group = f.create_group("/particles")
    allp = h5md.all_particles = h5md.particles_group.create_group("all")
    n = int(config.n_particles)
    indices = np.asarray(indices)
    allp.create_dataset("mass", (n,), dtype)[...] = config.mass
    if charges is not False:
        allp.create_dataset("charge", (n,), dtype="float32")[indices] = charges
    if dielectrics is not False:
        allp.create_dataset("dielectric", (n,), dtype="float32")[indices] = dielectrics
    box = allp.create_group("box")
    box.attrs["dimension"] = 3
    box.attrs["boundary"] = np.array([np.bytes_(s) for s in 3 * ["periodic"]], dtype="S8")
    n_frames = n_output_frames(int(config.n_steps), int(config.n_print))
    species = allp.create_dataset("species", (n,), dtype="i")
    _, h5md.positions_step, h5md.positions_time, h5md.positions = setup_time_dependent_element(
        "position", allp, n_frames, (n, 3), dtype, units="nm")
    if velocity_out:
        (_, h5md.velocities_step, h5md.velocities_time,
         h5md.velocities) = setup_time_dependent_element(
            "velocity", allp, n_frames, (n, 3), dtype, units="nm ps-1")
    if force_out:
        _, h5md.forces_step, h5md.forces_time, h5md.forces = setup_time_dependent_element(
            "force", allp, n_frames, (n, 3), dtype, units="kJ mol-1 nm-1")
    for attr, name, shape, dt, unit in _observables(dtype, charges, plumed_out):
        _, st, tm, val = setup_time_dependent_element(name, h5md.observables, n_frames, shape,
                                                      dt, units=unit)
        setattr(h5md, attr + "_step", st)
        setattr(h5md, attr + "_time", tm)
        setattr(h5md, attr, val)
    _, h5md.box_step, h5md.box_time, h5md.box_value = setup_time_dependent_element(
        "edges", box, n_frames, (3, 3), "float32", units="nm")
    n2t = _name_to_type(config)
    order = np.argsort(indices)
    names = np.asarray(names)
    for i in order:
        nm = names[i].decode("utf-8") if isinstance(names[i], bytes) else str(names[i])
        species[indices[i]] = n2t[nm]
    h5md.parameters.attrs["config.toml"] = np.bytes_(str(config))
    vmd = h5md.parameters.create_group("vmd_structure")
    vmd.create_dataset("indexOfSpecies", (config.n_types,), "i")[:] = np.arange(config.n_types)
    # VMD's h5md plugin reads at most 16 characters of a name
    name_ds = vmd.create_dataset("name", (config.n_types,), "S16")
    type_ds = vmd.create_dataset("type", (config.n_types,), "S16")
    resid = None
    if molecules is not None:
        resid = vmd.create_dataset("resid", (n,), "i")
    for i, nm in config.type_to_name_map.items():
        name_ds[i] = np.bytes_(nm[:16])
        type_ds[i] = np.bytes_("solvent" if nm == "W" else "membrane")
    a1 = np.asarray(bonds_2_atom1, dtype=np.int64)
    a2 = np.asarray(bonds_2_atom2, dtype=np.int64)
    bfrom = vmd.create_dataset("bond_from", (len(a1),), "i")
    bto = vmd.create_dataset("bond_to", (len(a1),), "i")
    if len(a1):
        bfrom[:] = indices[a1] + 1
        bto[:] = indices[a2] + 1
    if resid is not None:
        resid[indices[order]] = molecules


# float64 copies of a frame's particle arrays, kept between frames (fresh
# allocations of this size are mapped anew each time and fault in page by
# page); one set per thread, since trajectory writer threads call store_data
_F64_SCRATCH = threading.local()


def _as_f64(x, slot):
    bufs = getattr(_F64_SCRATCH, "bufs", None)
    if bufs is None:
        bufs = _F64_SCRATCH.bufs = {}
    buf = bufs.get(slot)
    if buf is None or buf.shape != x.shape:
        buf = bufs[slot] = np.empty(x.shape, dtype=np.float64)
    np.copyto(buf, x)
    return buf


def store_data(h5md, step, frame, indices, positions, velocities, forces, box_size, temperature,
               pressure, kinetic_energy, bond2_energy, bond3_energy, bond4_energy, field_energy,
               field_q_energy, plumed_bias, time_step, config, velocity_out=False,
               force_out=False, charge_out=False, plumed_out=False, dump_per_particle=False,
               comm=None):
    """One output frame (hymd/file_io.py:527-779): step and time of every
    element, the particle data in index order, energies, the momentum,
    angular momentum and torque sums, temperature, pressure, box edges and
    the thermostat work; then the reference's one-line energy log."""
    t = step * time_step
    steps = [h5md.positions_step, h5md.total_energy_step, h5md.potential_energy_step,
             h5md.kinetc_energy_step, h5md.bond_energy_step, h5md.angle_energy_step,
             h5md.dihedral_energy_step, h5md.field_energy_step, h5md.total_momentum_step,
             h5md.angular_momentum_step, h5md.torque_step, h5md.temperature_step,
             h5md.pressure_step, h5md.box_step, h5md.thermostat_work_step]
    times = [h5md.positions_time, h5md.total_energy_time, h5md.potential_energy_time,
             h5md.kinetc_energy_time, h5md.bond_energy_time, h5md.angle_energy_time,
             h5md.dihedral_energy_time, h5md.field_energy_time, h5md.total_momentum_time,
             h5md.angular_momentum_time, h5md.torque_time, h5md.temperature_time,
             h5md.pressure_time, h5md.box_time, h5md.thermostat_work_time]
    if velocity_out:
        steps.append(h5md.velocities_step)
        times.append(h5md.velocities_time)
    if force_out:
        steps.append(h5md.forces_step)
        times.append(h5md.forces_time)
    if charge_out:
        steps.append(h5md.field_q_energy_step)
        times.append(h5md.field_q_energy_time)
    if plumed_out:
        steps.append(h5md.plumed_bias_step)
        times.append(h5md.plumed_bias_time)
    for d in steps:
        d[frame] = step
    for d in times:
        d[frame] = t
    indices = np.asarray(indices)
    positions = np.asarray(positions)
    velocities = np.asarray(velocities)
    forces = np.asarray(forces)
    # the reference sorts the rows by global index before a fancy-indexed
    # write; rows that already hold consecutive ascending indices (one GPU
    # holding the whole system, in the caller's order) are a plain slice
    n_loc = indices.shape[0]
    if n_loc and np.array_equal(indices, np.arange(indices[0], indices[0] + n_loc)):
        rows = slice(int(indices[0]), int(indices[0]) + n_loc)
        put = lambda dset, x: dset.__setitem__((frame, rows), x)  # noqa: E731
    else:
        order = np.argsort(indices)
        put = lambda dset, x: dset.__setitem__((frame, indices[order]), x[order])  # noqa: E731
    put(h5md.positions, positions)
    if velocity_out:
        put(h5md.velocities, velocities)
    if force_out:
        put(h5md.forces, forces)
    if charge_out:
        h5md.field_q_energy[frame] = field_q_energy
    if plumed_out:
        h5md.plumed_bias[frame] = plumed_bias
    potential = bond2_energy + bond3_energy + bond4_energy + field_energy + field_q_energy
    # sums over particles in float64 (the reference adds float32 arrays in
    # float32); sum(a x b) from column dot products, without the N x 3 cross
    p64, v64, f64 = (_as_f64(x, k) for k, x in enumerate((positions, velocities, forces)))
    p = [p64[:, d] for d in range(3)]
    v = [v64[:, d] for d in range(3)]
    fc = [f64[:, d] for d in range(3)]

    def cross_sum(a, b):
        return np.array([np.dot(a[1], b[2]) - np.dot(a[2], b[1]),
                         np.dot(a[2], b[0]) - np.dot(a[0], b[2]),
                         np.dot(a[0], b[1]) - np.dot(a[1], b[0])])

    total_momentum = config.mass * np.array([np.sum(v[d]) for d in range(3)])
    angular_momentum = config.mass * cross_sum(p, v)
    torque = config.mass * cross_sum(p, fc)
    total = kinetic_energy + potential
    h5md.total_energy[frame] = total
    h5md.potential_energy[frame] = potential
    h5md.kinetc_energy[frame] = kinetic_energy
    h5md.bond_energy[frame] = bond2_energy
    h5md.angle_energy[frame] = bond3_energy
    h5md.dihedral_energy[frame] = bond4_energy
    h5md.field_energy[frame] = field_energy
    h5md.total_momentum[frame, :] = total_momentum
    h5md.angular_momentum[frame, :] = angular_momentum
    h5md.torque[frame, :] = torque
    h5md.temperature[frame] = temperature
    h5md.pressure[frame] = pressure
    for d in range(3):
        h5md.box_value[frame, d, d] = box_size[d]
    h5md.thermostat_work[frame] = config.thermostat_work
    _log_frame(step, time_step, temperature, total, kinetic_energy, potential, field_energy,
               field_q_energy, bond2_energy, bond3_energy, bond4_energy, plumed_bias,
               total_momentum, config, dump_per_particle)


def _log_frame(step, time_step, temperature, total, kinetic, potential, field, field_q, bond,
               angle, dihedral, bias, momentum, config, dump_per_particle):
    """The energy table line of hymd/file_io.py:716-779: only nonzero energy
    columns, the conserved-quantity drift when an initial energy is set."""
    names = ["step", "time", "temp", "tot E", "kin E", "pot E", "field E", "elec E", "bond E",
             "ang E", "dih E", "bias E", "Px", "Py", "Pz",
             "ΔH" if config.target_temperature else "ΔE"]
    keep = np.ones(len(names), bool)
    keep[6:12] = np.array([field, field_q, bond, angle, dihedral, bias]) != 0.0
    initial = getattr(config, "initial_energy", None)
    if initial is None:
        names[-1] = ""
    div = 1.0
    if dump_per_particle:
        for i in range(3, 9):
            names[i] = names[i][:-2] + "E/N"
        names[-1] += "/N"
        div = config.n_particles
    drift = 0.0
    if initial is not None:
        drift = total - initial - (config.thermostat_work if config.target_temperature else 0.0)
    vals = [step, time_step * step, temperature, total / div, kinetic / div, potential / div,
            field / div, field_q / div, bond / div, angle / div, dihedral / div, bias / div,
            momentum[0] / div, momentum[1] / div, momentum[2] / div, drift / div]
    cols = [i for i in range(len(names)) if keep[i]]
    header = "".join("{:>13}".format(names[i]) for i in cols)
    data = "{:13}".format(vals[cols[0]]) + "".join("{:13.5g}".format(vals[i]) for i in cols[1:])
    log.info("\n%s\n%s", header, data)


def distribute_input(in_file, rank, size, n_particles, max_molecule_size=201, comm=None):
    """Contiguous index ranges of the input arrays per rank, never splitting
    a molecule (hymd/file_io.py:781-874): with `molecules` in the input, each
    rank's nominal boundary n_per_rank * (rank + 1) is moved to the first
    molecule break at or after it (a window of max_molecule_size + 2 extra
    entries is read around it).  With one process (the GPU path) rank = 0,
    size = 1 gives the whole range.  Returns (list of indices, molecules
    present)."""
    if n_particles is None:
        n_particles = len(in_file["indices"])
    per = n_particles // size
    has_mol = "molecules" in in_file
    if not has_mol:
        lo = rank * per
        hi = n_particles if rank == size - 1 else (rank + 1) * per
        return list(range(lo, hi)), False
    extra = max_molecule_size + 2
    extra = extra if per > extra else per
    if rank == 0:
        lo = 0
        hi = n_particles if size == 1 else (rank + 1) * per + extra
    elif rank == size - 1:
        lo, hi = rank * per - 1, n_particles
    else:
        lo, hi = rank * per - 1, (rank + 1) * per + extra
    mol = np.asarray(in_file["molecules"][lo:hi])
    idx = np.asarray(in_file["indices"][lo:hi])
    ends = np.nonzero(np.diff(mol))[0]  # last position of each molecule in the window
    if rank == 0:
        first = 0
        last = n_particles if size == 1 else idx[ends[ends >= per][0] + 1]
    elif rank == size - 1:
        first = idx[ends[ends > 0][0]] + 1
        last = n_particles
    else:
        first = idx[ends[ends > 0][0]] + 1
        last = idx[ends[ends > per][0]] + 1
    return list(range(int(first), int(last))), True
