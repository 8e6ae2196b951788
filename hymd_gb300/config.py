"""Simulation configuration (the fields of hymd/input_parser.py:159-211 that the
hybrid particle-field force path reads).

Only the semantics that the force path depends on are mirrored:
  * ``time_step`` is the INNER rRESPA step; the outer step is
    ``respa_inner * time_step`` (hymd/main.py:802-806).
  * ``mesh_size`` is an int or a triple; ``box_size`` is stored as float32
    values (hymd/input_parser.py:736) but handed to kernels as float64.
  * ``m`` holds the per-type paint masses (default 1.0), ``mass`` the single
    particle mass used by the integrator (default 72).
  * without a barostat, ``rho0 = a = N / V`` (hymd/hamiltonian.py:41-47).
"""
from dataclasses import dataclass, field
from typing import ClassVar, List, Optional, Union

import numpy as np


@dataclass
class Config:
    gas_constant: ClassVar[float] = 0.0083144621  # kJ mol-1 K-1
    coulomb_constant: ClassVar[float] = 138.935458  # kJ nm mol-1 e-2

    n_steps: int
    time_step: float
    mesh_size: Union[List[int], np.ndarray, int]
    sigma: float
    kappa: float

    dtype: Optional[type] = None
    box_size: Union[List[float], np.ndarray, None] = None
    n_print: Optional[int] = None
    tau: Optional[float] = None
    start_temperature: Union[float, bool, None] = None
    target_temperature: Union[float, bool, None] = None
    mass: Optional[float] = None
    hamiltonian: Optional[str] = None
    respa_inner: int = 1
    bonds: list = field(default_factory=list)
    angle_bonds: list = field(default_factory=list)
    dihedrals: list = field(default_factory=list)
    chi: list = field(default_factory=list)
    n_particles: Optional[int] = None
    thermostat_coupling_groups: List[List[str]] = field(default_factory=list)
    thermostat_work: float = 0.0
    cancel_com_momentum: Union[int, bool] = False
    coulombtype: Optional[str] = None
    dielectric_const: Optional[float] = None
    # PIC_Spectral_GPE (hymd/input_parser.py:194-198): per-type relative
    # dielectric values indexed by type id (as sort_dielectric_by_type_id
    # leaves them), convergence measure, polarisation mixing, tolerance
    dielectric_type: list = field(default_factory=list)
    convergence_type: Optional[str] = None
    pol_mixing: Optional[float] = None
    conv_crit: Optional[float] = None
    self_energy: Optional[float] = None
    type_charges: Union[List[float], np.ndarray, None] = None
    rho0: Optional[float] = None
    a: Optional[float] = None
    pressure: bool = False
    barostat: Optional[str] = None
    barostat_type: Optional[str] = None
    tau_p: Optional[float] = None
    target_pressure: object = None
    n_b: Optional[int] = None
    m: List[float] = field(default_factory=list)
    n_types: Optional[int] = None
    unique_names: Optional[list] = None
    type_to_name_map: Optional[dict] = None

    def mesh(self):
        """Mesh dimensions as a 3-tuple of ints."""
        n = np.asarray(self.mesh_size, dtype=np.int64).reshape(-1)
        if n.size == 1:
            n = np.repeat(n, 3)
        return tuple(int(x) for x in n)

    def box(self):
        return np.asarray(self.box_size, dtype=np.float64).reshape(3)

    def volume(self):
        return float(np.prod(self.box()))


@dataclass
class Target_pressure:
    P_L: Union[bool, float]
    P_N: Union[bool, float]
