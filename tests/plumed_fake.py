"""A PLUMED kernel stand-in for the tests (py-plumed and the PLUMED library
are not installed): the `cmd` protocol of PLUMED's Python/C API with the
four actions of the reference's PLUMED test input (test/test_plumed.py):

    d14: DISTANCE ATOMS=1,4            distance of two atoms (1-based global
                                       indices), minimum image in the box
    RESTRAINT ARG=d14 KAPPA=k AT=a     bias 1/2 k (d - a)^2, forces -dE/dx
    DUMPATOMS ATOMS=1-N FILE=f         xyz frame: N, the box diagonal, "X x y z"
    PRINT ARG=d14 FILE=f               "#! FIELDS time d14" then "time value"

Forces are added into the array given by setForces (PLUMED's convention),
the bias goes to getBias.  Checked against the reference's PLUMED outputs
(refforces.txt, refDIST, reftestdump.xyz, the bias 635.5621691482) in
tests/test_plumed.py.
"""
import numpy as np


class _Local:
    """local[g]: the row of global index g."""

    def __init__(self, inv):
        self.inv = inv

    def __getitem__(self, g):
        return int(self.inv[g])


class FakePlumed:
    def __init__(self):
        self.p = {}
        self.actions = []
        self.calls = []
        self.files = {}
        self.needs_energy = False

    def _parse(self, path):
        for line in open(path):
            line = line.strip()
            if not line:
                continue
            label = None
            if ":" in line.split()[0]:
                label, line = line.split(":", 1)
                line = line.strip()
            words = line.split()
            kw = dict(w.split("=", 1) for w in words[1:] if "=" in w)
            self.actions.append((words[0], label, kw))

    def cmd(self, name, val=None):
        self.calls.append(name)
        if name == "getApiVersion":
            val[0] = 9
        elif name == "setPlumedDat":
            self._parse(val)
        elif name in ("setMDEngine", "setLogFile", "setTimestep", "setNatoms", "setKbT",
                      "setAtomsNlocal", "setAtomsGatindex", "setStep", "setForces",
                      "setPositions", "setCharges", "setMasses", "setBox", "setEnergy"):
            self.p[name] = val
        elif name == "isEnergyNeeded":
            val[0] = 1 if self.needs_energy else 0
        elif name == "performCalc":
            self._calc()
        elif name == "getBias":
            val[0] = self.bias
        elif name in ("setNoVirial", "init", "prepareCalc"):
            pass
        else:
            raise ValueError(f"unknown PLUMED command {name}")

    def _calc(self):
        n = int(self.p["setAtomsNlocal"])
        gat = np.asarray(self.p["setAtomsGatindex"])
        x = np.asarray(self.p["setPositions"]).reshape(n, 3)
        f = self.p["setForces"].reshape(n, 3)  # a view: PLUMED adds into it
        box = np.diag(np.asarray(self.p["setBox"]).reshape(3, 3))
        # local row of a global index (an inverse array: the runs hold up to
        # millions of atoms)
        inv = np.full(int(gat.max()) + 1 if n else 1, -1, dtype=np.int64)
        inv[gat] = np.arange(n)
        local = _Local(inv)
        step = int(self.p["setStep"])
        time = step * float(self.p["setTimestep"])
        values, grads = {}, {}
        self.bias = 0.0
        for kind, label, kw in self.actions:
            if kind == "DISTANCE":
                a, b = (int(s) - 1 for s in kw["ATOMS"].split(","))
                d = x[local[b]] - x[local[a]]
                d -= box * np.round(d / box)
                r = float(np.sqrt(d @ d))
                values[label] = r
                grads[label] = {a: -d / r, b: d / r}
            elif kind == "RESTRAINT":
                arg = kw["ARG"]
                k, at = float(kw["KAPPA"]), float(kw["AT"])
                dv = values[arg] - at
                self.bias += 0.5 * k * dv * dv
                for g, gr in grads[arg].items():
                    f[local[g]] -= k * dv * gr
            elif kind == "PRINT":
                fh = self._file(kw["FILE"], "#! FIELDS time " + " ".join(kw["ARG"].split(",")))
                fh.write(" {:.6f} ".format(time)
                         + " ".join("{:.6f}".format(values[a]) for a in kw["ARG"].split(","))
                         + "\n")
            elif kind == "DUMPATOMS":
                lo, hi = (int(s) for s in kw["ATOMS"].split("-"))
                fh = self._file(kw["FILE"], None)
                fh.write(f"{hi - lo + 1}\n")
                fh.write(" " + " ".join("{:.6f}".format(b) for b in box) + "\n")
                for g in range(lo - 1, hi):
                    fh.write("X " + " ".join("{:.6f}".format(c) for c in x[local[g]]) + "\n")
        for fh in self.files.values():
            fh.flush()

    def _file(self, path, header):
        if path not in self.files:
            self.files[path] = open(path, "w")
            if header:
                self.files[path].write(header + "\n")
        return self.files[path]

    def finalize(self):
        for fh in self.files.values():
            fh.close()
        self.files = {}
