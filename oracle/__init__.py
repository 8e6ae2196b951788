"""CPU oracle for the hPF force path -- TEST INFRASTRUCTURE ONLY.

This package restates, in FP64 numpy and plain C, what HyMD computes on the
hybrid particle-field force path.  It is the checker for the CUDA library in
``hymd_gb300``: only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` import it.  The
product path never imports, links or executes anything here.

Modules
-------
field      paint / filter / external potential / gradient / readout / energy /
           PIC_Spectral electrostatics / pressure   (hymd/field.py, hymd/pressure.py)
bonded     ctypes wrapper over libbonded_oracle.so, the C restatement of the
           f2py Fortran kernels cbf/caf/cdf (+ _d variants)   (hymd/*.f90)
hamiltonian quadratic restatement of SquaredPhi / DefaultNoChi / DefaultWithChi
           (hymd/hamiltonian.py)
md         the rRESPA outer/inner loop of hymd/main.py:802-1169 on the oracle

Parity pins: see tests/golden/ (fixtures generated from the reference's own
Python modules and its test files) and tests/test_oracle_*.py.
"""
