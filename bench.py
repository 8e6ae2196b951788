"""Benchmark: MD steps/s and ns/day of the hybrid particle-field rRESPA step.

Workload (default): the 500k-bead charged-peptide system -- 200 chains of 50
residues (backbone + side chain, harmonic bonds, 120-degree angles, cosine +
combined bending-torsion dihedrals), 20% of side chains charged +-1 e with
counter-ions, W solvent to 500 000 beads, box 40 nm, mesh 128^3, 3 types,
PIC_Spectral electrostatics (eps_r 80), CSVR thermostat at 323 K,
time_step 0.03 ps, respa_inner 10.  One step = one outer rRESPA step (10
inner bonded steps + the density and charge field evaluations), run from a
CUDA graph.  Inputs (the system state) are resident in HBM; L2 is flushed
between timed steps (a 256 MB write, then a 256 MB read so that the evicted
lines are clean), outside the per-step CUDA-event windows.  --workload
melt10k / membrane162k select the other two single-system configurations.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl hpf|reference]

--impl reference times the CPU restatement of the same step (oracle/cpu_md.py:
FP32, the reference's order of operations, OpenMP + threaded FFTs over all
host cores; the reference's own CPU code cannot be built here or on the GPU
box).  N > 1 (torchrun): independent replicas, one per GPU; value = sum over
ranks.
"""
import argparse
import copy
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MD steps/s & ns/day per GB300 vs plain GPU form at <=1e-5 force rel-RMS vs FP64"
WORKLOAD = "peptide500k"

# workload -> description and coupling (thermostat / barostat)
WORKLOADS = {
    "membrane162k": ("lipid membrane 162k beads (6000 x 12-bead lipids + 90k W), box 27 nm, "
                     "mesh 64^3, 5 types",
                     dict(thermostat=True, barostat="isotropic"),
                     "NPT: SCR barostat (isotropic, 1 bar, tau_p 1 ps, every step) + "
                     "CSVR thermostat (323 K, tau 0.1 ps)"),
    "melt10k": ("binary homopolymer melt 10k beads (1000 x 10-bead chains), box 10 nm, "
                "mesh 32^3, 2 types",
                dict(thermostat=True, barostat=None), "NVT: CSVR thermostat (323 K, tau 0.1 ps)"),
    "peptide500k": ("charged peptides 500k beads (200 x 50-residue BB+SC chains, 20% charged "
                    "side chains + counter-ions, W), box 40 nm, mesh 128^3, 3 types, "
                    "PIC_Spectral eps_r 80, CBT dihedrals",
                    dict(thermostat=True, barostat=None),
                    "NVT: CSVR thermostat (323 K, tau 0.1 ps)"),
}


def max_over_ranks(x, ws, device):
    """The largest of the ranks' values of x (a timed region's duration: the
    whole job is as slow as its slowest rank); x itself on one rank.  The
    process group is NCCL in the GPU arm, gloo in the CPU tests."""
    if ws <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def _config_block(cfg, n, workload=WORKLOAD, extra=None):
    desc, _, ensemble = WORKLOADS[workload]
    d = {"workload": desc, "n_beads": int(n), "mesh": list(cfg.mesh()), "respa_inner": int(cfg.respa_inner),
         "time_step_ps": float(cfg.time_step), "sigma": cfg.sigma, "kappa": cfg.kappa,
         "l2": "flushed between timed steps (256 MB write, then 256 MB read so the evicted "
               "lines are clean; outside the timed windows)",
         "parallelism": "replicas only", "ensemble": ensemble}
    if extra:
        d.update(extra)
    return d


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region (the raw
    samples go to BENCH_CLOCK_DIR, default the system temp directory; the
    JSON line carries their summary)."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        d = os.environ.get("BENCH_CLOCK_DIR") or tempfile.gettempdir()
        self.path = os.path.join(d, f"clocks_bench_{os.getpid()}.csv")

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _traffic(workload):
    """Per-launch DRAM bytes (read + write) of the step's kernels from one ncu
    capture of this workload, if recorded under profiles/."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if not os.path.exists(p):
        return {}
    return json.load(open(p)).get(workload, {})


def cpu_step(sys_, seed=0):
    """The FP32 multi-core CPU restatement of one outer step (oracle/cpu_md.py)
    on the workload's own system, with the same thermostat."""
    from oracle import cpu_md
    from oracle import hamiltonian as oh
    fun = oh.functional_of_config(sys_["config"])
    return cpu_md.CpuStep(sys_, fun.Q, fun.b, workers=os.cpu_count() or 1, seed=seed)


def cpu_baseline(sys_, steps=2, budget_s=60.0):
    """A bounded sample of the CPU step: one untimed step, then up to `steps`
    timed steps within `budget_s` seconds.  Returns (steps/s, seconds, done,
    threads)."""
    from oracle import cpu_md
    cs = cpu_step(sys_)
    cs.step()
    t0 = time.perf_counter()
    done = 0
    while done < max(1, steps) and (done == 0 or time.perf_counter() - t0 < budget_s):
        cs.step()
        done += 1
    dt = time.perf_counter() - t0
    return done / dt, dt, done, cpu_md.threads()


def run_reference(args):
    ws, rank = _dist()
    if rank != 0:
        return 0
    from hymd_gb300 import systems
    s = systems.BUILDERS[args.workload](seed=2)
    cfg = s["config"]
    from oracle import cpu_md
    cs = cpu_step(s)
    t0 = time.perf_counter()
    for _ in range(max(1, args.warmup)):
        cs.step()
        if time.perf_counter() - t0 > 30.0:
            break
    # bounded sample: K steps, at most ~90 s of host work
    t0 = time.perf_counter()
    done = 0
    while done < max(1, args.steps) and (done == 0 or time.perf_counter() - t0 < 90.0):
        cs.step()
        done += 1
    secs = time.perf_counter() - t0
    sps = done / secs
    threads = cpu_md.threads()
    ns_day = sps * cfg.respa_inner * cfg.time_step * 86400 / 1000.0
    line = {"impl": "reference", "metric": METRIC, "value": sps, "unit": "steps/s",
            "n_gpus": ws, "steps": done, "warmup": args.warmup,
            "ms_per_step": 1000.0 / sps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "ns_per_day": ns_day,
            "config": _config_block(cfg, len(s["positions"]), args.workload),
            "cpu_baseline": {"value": sps, "unit": "steps/s", "cores": threads, "kind": "port",
                             "sample": f"{done} outer steps of the full workload ({secs:.1f} s) "
                                       "on the FP32 restatement of the reference's step "
                                       f"(oracle/cpu_md.py): OpenMP over {threads} threads, "
                                       f"FFTs over {os.cpu_count()} workers; restatement, "
                                       "not the reference"},
            "e2e": {"value": sps, "unit": "steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


class L2Flush:
    """Evicts L2 (129 MB) between timed steps: a 256 MB write, then a 256 MB
    read, so that the lines left in L2 are clean and the next step's misses
    do not first write back the flush's own data."""

    def __init__(self, torch, dev):
        self.w = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
        self.r = torch.ones(64 * 1024 * 1024, dtype=torch.float32, device=dev)
        self.sink = torch.empty(1, dtype=torch.float32, device=dev)

    def zero_(self):
        self.w.zero_()
        self.sink.copy_(self.r.sum().reshape(1))


def step_breakdown(md, flush, torch, reps=10):
    """Per-stage device time of one MD step (diagnostic, printed to stderr):
    the fused rRESPA kernel timed as a captured graph, the field step by
    hpf_field_step_profile (CUDA events between its stages), the thermostat
    scaling as a graph.  L2 is flushed before each timed stage group (which
    also keeps the GPU busy while the host enqueues the stages)."""
    from hymd_gb300 import _lib
    st = torch.cuda.current_stream()

    def graph(fn):
        s = torch.cuda.Stream()
        s.wait_stream(st)
        with torch.cuda.stream(s):
            fn()
        st.wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            fn()
        return g

    # the stages are replayed out of order (the inner loop without the field
    # step, the field step with its own paint): snapshot the physical state
    # and put it back afterwards, with one field step to clear the paint's
    # accumulators
    keep = {k: getattr(md, k).clone() for k in ("r", "v", "f_b", "f_field", "f_elec", "state",
                                                "counter", "field_sums")
            if getattr(md, k, None) is not None}
    box0 = md.box_now()
    thermo = md.thermo_args is not None
    g_respa = graph(lambda: md._inner_fused(_lib.stream_ptr()))
    g_scale = graph(lambda: _lib.call("hpf_csvr_scale", _lib.ptr(md.v), _lib.ptr(md.group),
                                      md.n, _lib.ptr(md.state),
                                      int(md.thermo_args.remove_com) if thermo else 1,
                                      _lib.stream_ptr()))
    fused = md.pm.spectral == "fused"
    # with the fused spectral passes, the profile's second stage holds all
    # three passes (accumulators -> force mesh) and the next two are empty
    names = ["respa", "paint", "spectral_fused" if fused else "r2c", "kspace", "c2r",
             "readout_kick", "thermostat_scale"]
    tot = {k: 0.0 for k in names}
    # the fused kernel with its data left in L2 (back-to-back replays), for
    # comparison with the flushed figure
    flush.zero_()
    g_respa.replay()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(reps):
        g_respa.replay()
    b.record(st)
    b.synchronize()
    tot["respa_l2_resident"] = a.elapsed_time(b) * 1000.0 / reps
    us = (_lib.ctypes.c_float * 5)()
    for _ in range(reps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        g_respa.replay()
        b.record(st)
        b.synchronize()
        tot["respa"] += a.elapsed_time(b) * 1000.0 / reps
        scale = md.state.data_ptr() + 12 * 8 if md.baro_args is not None else None
        # the flush also keeps the GPU busy while the host enqueues the
        # stages, so the events see no host launch gaps
        flush.zero_()
        _lib.call("hpf_field_step_profile", md.pm._h, _lib.ptr(md.r), _lib.ptr(md.types), md.n,
                  md.masses, _lib.ptr(md.f_field), _lib.ptr(md.field_sums),
                  None if scale is None else _lib.ctypes.c_void_p(scale),
                  md._kick_args(thermo), _lib.stream_ptr(), us)
        for k, x in zip(names[1:6], us):
            tot[k] += x / reps
    if fused:
        del tot["kspace"], tot["c2r"]
    for _ in range(reps):
        flush.zero_()
        a.record(st)
        g_scale.replay()
        b.record(st)
        b.synchronize()
        tot["thermostat_scale"] += a.elapsed_time(b) * 1000.0 / reps
    if md.charges is not None:
        # the charge path of the step (paint of the charged beads, transforms
        # with the Poisson map, readout of q E), without the kick it carries
        # in the step
        g_pic = graph(lambda: _lib.call(
            "hpf_pic_step_list", md.pm._h, _lib.ptr(md.r), _lib.ptr(md.charges),
            _lib.ptr(md.charged), md.charged.numel(), md.n, float(md.elec_factor),
            _lib.ptr(md.f_elec), None, None, _lib.stream_ptr()))
        tot["pic"] = 0.0
        for _ in range(reps):
            flush.zero_()
            a.record(st)
            g_pic.replay()
            b.record(st)
            b.synchronize()
            tot["pic"] += a.elapsed_time(b) * 1000.0 / reps
    torch.cuda.synchronize()
    md.pm.set_box(box0)
    for k, t in keep.items():
        getattr(md, k).copy_(t)
    md._field(_lib.stream_ptr(), torch.zeros_like(md.field_sums))  # clears the accumulators
    for k in ("r", "f_field", "f_elec", "field_sums"):
        if k in keep:
            getattr(md, k).copy_(keep[k])
    torch.cuda.synchronize()
    return tot


def adjoint_cost(md, flush, torch, reps=10):
    """Device time (us) of one forward field-force evaluation (hpf_field_step:
    paint, r2c, k-space, c2r, readout) against the adjoint (hpf_field_adjoint)
    giving dW/d(chi, kappa, sigma), and with dW/dx as well; each as a captured
    graph, L2 flushed before each repetition."""
    from hymd_gb300 import _lib
    st = torch.cuda.current_stream()
    T = md.T
    sums = torch.zeros(T * (T + 1) // 2 + 1 + T, dtype=torch.float64, device=md.r.device)
    grad = torch.empty_like(md.r)
    f = torch.empty_like(md.r)

    def fwd():
        _lib.call("hpf_field_step", md.pm._h, _lib.ptr(md.r), _lib.ptr(md.types), md.n, md.masses,
                  _lib.ptr(f), None, None, None, _lib.stream_ptr())

    def adj(with_x):
        def fn():
            _lib.call("hpf_field_adjoint", md.pm._h, _lib.ptr(md.r), _lib.ptr(md.types), md.n,
                      md.masses, _lib.ptr(grad) if with_x else None, _lib.ptr(sums),
                      _lib.stream_ptr())
        return fn

    out = {}
    for name, fn in (("forward_force_us", fwd), ("dW_dparams_us", adj(False)),
                     ("dW_dx_and_params_us", adj(True))):
        s = torch.cuda.Stream()
        s.wait_stream(st)
        with torch.cuda.stream(s):
            fn()
        st.wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            fn()
        tot = 0.0
        for _ in range(reps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            g.replay()
            b.record(st)
            b.synchronize()
            tot += a.elapsed_time(b) * 1000.0 / reps
        out[name] = tot
    out["params_over_forward"] = out["dW_dparams_us"] / out["forward_force_us"]
    return out


def accuracy(md, sys_, ham, torch):
    """Errors of the state the timed region left, against the FP64 oracle:
    the field and electrostatic forces, field energy, electrostatic energy
    and pressure vector through the drop-in API (hymd_gb300.field /
    pressure, a fresh mesh context) and the bonded forces of the fused plan
    (hpf_respa_forces) against the real(8) C restatement of the Fortran
    kernels, all at the positions and velocities of the last timed step."""
    from hymd_gb300 import _lib
    from hymd_gb300 import field as gf
    from hymd_gb300.pressure import comp_pressure
    from oracle import bonded as ob
    from oracle import field as of
    from oracle import hamiltonian as oh
    of.FFT_WORKERS = os.cpu_count() or 1
    # the state's own box (a barostat has moved it away from the config's)
    cfg = copy.copy(sys_["config"])
    cfg.box_size = md.box.cpu().numpy().astype(np.float64)
    T = cfg.n_types
    R, V, Ty = md.r, md.v, md.types
    pm, fl, ecl, cl = gf.initialize_pm(None, cfg)
    phi, phi_fourier, force_on_grid, v_ext_fourier, v_ext, phi_transfer, phi_lap = fl
    gf.update_field(phi, phi_lap, phi_transfer, None, force_on_grid, ham, pm, R, Ty, cfg, v_ext,
                    phi_fourier, v_ext_fourier, cfg.m)
    F = torch.zeros_like(R)
    gf.compute_field_force(None, R, force_on_grid, F, Ty, T)
    psi = phi_q = None
    Fq = None
    if md.charges is not None:
        phi_q, phi_q_fourier, psi, elec_field = ecl
        elec_field_fourier, psi_fourier = cl
        Fq = torch.zeros_like(R)
        gf.update_field_force_q(md.charges, phi_q, phi_q_fourier, psi, psi_fourier,
                                elec_field_fourier, elec_field, Fq, None, ham, pm, R, cfg)
    W, _, Wq = gf.compute_field_and_kinetic_energy(phi, phi_q, psi, V, ham, R, Ty, v_ext, cfg,
                                                   None)
    zero3 = np.zeros(3)
    P = comp_pressure(phi, phi_q, psi, ham, V, cfg, phi_fourier, phi_lap, phi_transfer, R,
                      zero3, zero3)
    fb = torch.zeros_like(R)
    if md.plan is not None:
        _lib.call("hpf_respa_forces", md.plan, _lib.ptr(R), _lib.ptr(fb), _lib.ptr(md.box), None,
                  _lib.ptr(md.err), _lib.stream_ptr())
    torch.cuda.synchronize()
    md.check_errors()
    pm.check_errors()

    # the oracle works in the caller's bead order
    r64 = md.in_input_order(R).cpu().numpy().astype(np.float64)
    v32 = md.in_input_order(V).cpu().numpy()
    types = sys_["types"]
    fun = oh.functional_of_config(cfg)
    ref = of.update_field(r64, types, T, cfg.mesh(), cfg.box(), cfg.m, fun, cfg.sigma)
    Fref = of.compute_field_force(ref["force_mesh"], r64, types, T, cfg.mesh(), cfg.box())

    def rel_rms(a, b):
        return float(np.sqrt(np.mean((np.asarray(a, np.float64) - b) ** 2))
                     / np.sqrt(np.mean(b ** 2)))

    out = {"reference": "FP64 oracle (oracle/field.py, pinned to the reference's own field.py "
                        "through tests/golden/field_ref.npz) at the last timed state",
           "force_rel_rms": rel_rms(md.in_input_order(F).cpu().numpy(), Fref)}
    Wref = of.field_energy(ref["phi"], fun, cfg.mesh(), cfg.box())
    out["energy_rel_err"] = abs(W - Wref) / abs(Wref)
    kw = {}
    if Fq is not None:
        q = sys_["charges"].astype(np.float64)
        qr = of.update_field_force_q(q, r64, cfg.mesh(), cfg.box(), cfg.sigma,
                                     cfg.dielectric_const)
        out["elec_force_rel_rms"] = rel_rms(md.in_input_order(Fq).cpu().numpy(), qr["forces"])
        es = float(cfg.self_energy or 0.0)
        Wq_ref = of.field_q_energy(qr["phi_q"], qr["psi"], es, cfg.mesh(), cfg.box())
        out["elec_energy_rel_err"] = abs(Wq - Wq_ref) / abs(Wq_ref)
        kw = dict(phi_q=qr["phi_q"], psi=qr["psi"], self_energy=es,
                  type_charges=list(cfg.type_charges))
    Pref = of.comp_pressure(ref["phi"], ref["phi_fourier"], fun, v32, cfg.mass, cfg.mesh(),
                            cfg.box(), cfg.sigma, zero3, zero3, **kw)
    out["pressure_rel_err"] = float(np.max(np.abs(P - Pref)) / np.max(np.abs(Pref[:6])))
    topo = sys_.get("topology")
    if md.plan is not None and topo is not None:
        (b2a, b2b, b2r, b2k, b3a, b3b, b3c, b3t, b3k, b4a, b4b, b4c, b4d, b4coeff, b4type,
         b4last) = topo
        box = cfg.box()
        fsum = np.zeros_like(r64)
        for fn, argv in ((ob.compute_bond_forces, (b2a, b2b, b2r, b2k)),
                         (ob.compute_angle_forces, (b3a, b3b, b3c, b3t, b3k))):
            if len(argv[0]):
                f = np.zeros_like(r64)
                fn(f, r64, box, *argv, precision="double")
                fsum += f
        if len(b4a):
            f = np.zeros_like(r64)
            nd = len(b4a)
            ob.compute_dihedral_forces(f, r64, np.zeros((nd, 4, 3)), np.zeros((nd, 6, 3, 3)), box,
                                       b4a, b4b, b4c, b4d, b4coeff, b4type, b4last, 0,
                                       precision="double")
            fsum += f
        bonded_beads = np.zeros(len(r64), bool)
        for idx in (b2a, b2b, b3a, b3b, b3c, b4a, b4b, b4c, b4d):
            bonded_beads[np.asarray(idx, np.int64)] = True
        got = md.in_input_order(fb).cpu().numpy()
        out["bonded_force_rel_rms"] = rel_rms(got[bonded_beads], fsum[bonded_beads])
        out["bonded_reference"] = "real(8) C restatement of cbf_d / caf_d / cdf_d"
    return out


def e2e_wall(md, flush, torch, steps):
    """Steps/s of RespaMD.run_host on the host wall clock: each step copies the
    positions and velocities in from page-locked host memory, runs the
    captured step and copies the positions out; time.perf_counter around the
    call and a synchronize, with the GPU idle at the start of each step (the
    L2 flush before it has finished)."""
    n = md.n
    r_h = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    v_h = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    r_out = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    r_h.copy_(md.r.cpu())
    v_h.copy_(md.v.cpu())
    md.run_host(r_h, v_h, r_out)
    torch.cuda.synchronize()
    tot = 0.0
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        md.run_host(r_h, v_h, r_out)
        torch.cuda.synchronize()
        tot += time.perf_counter() - t0
    if not torch.equal(r_out, md.r.cpu()):
        raise RuntimeError("end-to-end step: the positions read back differ from the device's")
    return steps / tot, 24 * n, 12 * n


def e2e_dropin(sys_, ham, torch, dev, steps):
    """Steps/s of a main.py-style outer step written with the drop-in calls
    (hymd/main.py:802-887, 975-1004, 1143-1169), numpy arrays in and out:
    positions and velocities copied in, integrate_velocity /
    integrate_position, compute_bond/angle/dihedral_forces for each inner
    step, update_field + compute_field_force + update_field_force_q, the
    second kick, positions and velocities copied out.  No thermostat (the
    reference's thermostat is host code outside the drop-in boundary).
    Host wall clock per step."""
    from hymd_gb300 import field as gf
    from hymd_gb300 import force as gfo
    from hymd_gb300.integrator import integrate_position, integrate_velocity
    cfg = sys_["config"]
    T = cfg.n_types
    n = len(sys_["positions"])
    mass = float(cfg.mass)
    dt, k = float(cfg.time_step), int(cfg.respa_inner)
    box_t = torch.as_tensor(cfg.box().astype(np.float32), device=dev)
    box = torch.as_tensor(cfg.box(), device=dev)  # device float64, as the kernels take it
    # term arrays on the device once, in the dtypes the entry points use
    # (int32 indices, float32 parameters), so no call converts them again
    real = {2, 3, 7, 8, 13}
    topo = [torch.as_tensor(np.asarray(x, np.float32 if i in real else np.int32), device=dev)
            for i, x in enumerate(sys_["topology"])]
    (b2a, b2b, b2r, b2k, b3a, b3b, b3c, b3t, b3k, b4a, b4b, b4c, b4d, b4coeff, b4type,
     b4last) = topo
    nd = b4a.numel()
    dip = torch.zeros((nd, 4, 3), dtype=torch.float32, device=dev)
    tr = torch.zeros((nd, 6, 3, 3), dtype=torch.float32, device=dev)
    types = torch.as_tensor(sys_["types"], device=dev)
    q = sys_.get("charges")
    Q = None if q is None else torch.as_tensor(q, device=dev)
    pm, fl, ecl, cl = gf.initialize_pm(None, cfg)
    phi, phi_fourier, force_on_grid, v_ext_fourier, v_ext, phi_transfer, phi_lap = fl
    z = lambda: torch.zeros((n, 3), dtype=torch.float32, device=dev)  # noqa: E731
    fb, fa, fdh, ff, fq = z(), z(), z(), z(), z()

    def bonded(r):
        fb.zero_(), fa.zero_(), fdh.zero_()
        gfo.compute_bond_forces(fb, r, box, b2a, b2b, b2r, b2k, sync=False)
        gfo.compute_angle_forces(fa, r, box, b3a, b3b, b3c, b3t, b3k, sync=False)
        if nd:
            gfo.compute_dihedral_forces(fdh, r, dip, tr, box, b4a, b4b, b4c, b4d, b4coeff,
                                        b4type, b4last, 0, sync=False)
        return fb + fa + fdh

    def field(r):
        gf.update_field(phi, phi_lap, phi_transfer, None, force_on_grid, ham, pm, r, types, cfg,
                        v_ext, phi_fourier, v_ext_fourier, cfg.m)
        gf.compute_field_force(None, r, force_on_grid, ff, types, T)
        if Q is not None:
            phi_q, phi_q_fourier, psi, elec_field = ecl
            elec_field_fourier, psi_fourier = cl
            gf.update_field_force_q(Q, phi_q, phi_q_fourier, psi, psi_fourier,
                                    elec_field_fourier, elec_field, fq, None, ham, pm, r, cfg)
            return ff + fq
        return ff.clone()

    r_np = np.ascontiguousarray(sys_["positions"], np.float32).copy()
    v_np = np.ascontiguousarray(sys_["velocities"], np.float32).copy()
    r = torch.as_tensor(r_np, device=dev)
    f_slow = field(r)
    f_bond = bonded(r)

    def step():
        nonlocal f_slow, f_bond
        r = torch.as_tensor(r_np, device=dev)
        v = torch.as_tensor(v_np, device=dev)
        v = integrate_velocity(v, f_slow / mass, k * dt)
        for _ in range(k):
            v = integrate_velocity(v, f_bond / mass, dt)
            r = torch.remainder(integrate_position(r, v, dt), box_t)
            f_bond = bonded(r)
            v = integrate_velocity(v, f_bond / mass, dt)
        f_slow = field(r)
        v = integrate_velocity(v, f_slow / mass, k * dt)
        r_np[...] = r.cpu().numpy()
        v_np[...] = v.cpu().numpy()

    for _ in range(3):
        step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    torch.cuda.synchronize()
    sps = steps / (time.perf_counter() - t0)
    pm.check_errors()
    return sps, 24 * n, 24 * n


def run_gpu(args):
    import torch

    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from hymd_gb300 import _lib, systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD

    s = systems.BUILDERS[args.workload](seed=2 + rank)
    cfg = s["config"]
    n = len(s["positions"])
    ham = get_hamiltonian(cfg)
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"],
                 charges=s.get("charges"), device=dev)
    # beads stored in mesh-cell order (a permutation; the physics is unchanged)
    md.sort_particles()
    # coupling of the workload (the membrane runs NPT: SCR barostat at 1 bar
    # every step and CSVR at 323 K); random numbers come from a seeded table
    md.couple(seed=100 + rank, n_steps=20000, **WORKLOADS[args.workload][1])
    md.prime()
    # two graphs per step (fused inner loop | field step + thermostat) so that
    # an event between them times the dominant kernel inside the timed region
    md.capture(split=True)
    flush = L2Flush(torch, dev)
    for _ in range(max(3, args.warmup)):
        md.run(1)
    torch.cuda.synchronize()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    st = torch.cuda.current_stream()
    evs = [tuple(torch.cuda.Event(enable_timing=True) for _ in range(3))
           for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for a, m, b in evs:
            flush.zero_()
            a.record(st)
            if md.graph_inner is not None:
                md.graph_inner.replay()
                m.record(st)
                md.graph_field.replay()
            else:
                md.graph.replay()
                m.record(st)
            b.record(st)
        torch.cuda.synchronize()
    barrier()
    ms = max_over_ranks(sum(a.elapsed_time(b) for a, m, b in evs), ws, dev)
    respa_ms = sum(a.elapsed_time(m) for a, m, b in evs) / args.steps
    ms_step = ms / args.steps
    sps = 1000.0 / ms_step
    md.check_errors()
    # accuracy of the state the timed region left (before any diagnostic runs)
    acc = accuracy(md, s, ham, torch) if rank == 0 and not args.no_accuracy else None

    # ---- the same K steps after 1000 more: the bead order of the setup sort
    # decays as the beads move (no re-sort, RespaMD.resort_every = 0)
    aged = None
    if not args.no_aging:
        md.run(1000)
        torch.cuda.synchronize()
        tot = 0.0
        for _ in range(args.steps):
            flush.zero_()
            a0, b0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a0.record(st)
            md.replay()
            b0.record(st)
            b0.synchronize()
            tot += a0.elapsed_time(b0)
        md.check_errors()
        tot = max_over_ranks(tot, ws, dev)
        aged = {"steps_before": args.warmup + args.steps + 1000,
                "value": 1000.0 * args.steps / tot * ws, "unit": "steps/s",
                "ms_per_step": tot / args.steps,
                "note": "the timed protocol of `value` after 1000 further steps, no re-sort"}

    # ---- end to end, host wall clock --------------------------------------
    e2e_sps, e2e_h2d, e2e_d2h = e2e_wall(md, flush, torch, args.steps)
    e2e_sps = 1.0 / max_over_ranks(1.0 / e2e_sps, ws, dev)  # the slowest rank's rate
    dropin = None
    if not args.no_dropin:
        d_sps, d_h2d, d_d2h = e2e_dropin(s, ham, torch, dev, max(3, min(args.steps, 20)))
        d_sps = 1.0 / max_over_ranks(1.0 / d_sps, ws, dev)
        dropin = {"value": d_sps * ws, "unit": "steps/s", "h2d_bytes_per_step": d_h2d,
                  "d2h_bytes_per_step": d_d2h,
                  "path": "main.py-style outer step over the drop-in calls (integrate_*, "
                          "compute_*_forces, update_field, compute_field_force, "
                          "update_field_force_q), numpy in / out, no thermostat, "
                          "host wall clock"}

    # ---- roofline -------------------------------------------------------------
    # dominant kernel: the fused rRESPA inner loop.  Algorithmic bytes are
    # those of the unfused inner step (read r, v, F; write r, v, F; bonded
    # term data: 72 N + 16 B + 20 A + 144 D) times respa_inner; the fused
    # kernel keeps the loop on chip, so its DRAM traffic is far lower.
    peak, peak_kind = _peaks()
    T = cfg.n_types
    M = int(np.prod(cfg.mesh()))
    Mc = cfg.mesh()[0] * cfg.mesh()[1] * (cfg.mesh()[2] // 2 + 1)
    topo = md.topo
    nb = topo.n_bonds if topo else 0
    na = topo.n_angles if topo else 0
    nd = topo.n_dihedrals if topo else 0
    respa_bytes = cfg.respa_inner * (72 * n + 16 * nb + 20 * na + 144 * nd)
    nq = int(md.charged.numel()) if md.charged is not None else 0
    fused_paint = md._paint_fused
    if fused_paint:
        # the launch also paints every bead (and the charged ones): the
        # paint's contract bytes, 16 N + 4 T M (+ 16 N_q + 4 M)
        respa_bytes += 16 * n + 4 * T * M + ((16 * nq + 4 * M) if nq else 0)
    respa_gbs = respa_bytes / (respa_ms * 1e-3) / 1e9
    traffic = _traffic(args.workload)
    # the other kernels of the step, timed stage by stage (graphs + events,
    # L2 flushed before each repetition)
    bd = step_breakdown(md, flush, torch)
    if args.breakdown and rank == 0:
        print(json.dumps({"breakdown_us": bd}), file=sys.stderr)
    adj = adjoint_cost(md, flush, torch)
    # algorithmic bytes per launch as the path's contract defines them (FP32
    # grids, cuFFT traffic excluded): paint reads r + type and writes T
    # grids; the k-space work reads T spectra and writes 3T; the readout
    # reads r + type and 3T grids once and writes F; the charge path of the
    # charged beads N_q is 44 N_q + 16 M + 32 Mc
    stage_bytes = {"paint": 16 * n + 4 * T * M, "kspace": 32 * T * Mc,
                   "spectral_fused": 32 * T * Mc,
                   "readout_kick": 28 * n + 12 * T * M,
                   "pic": 44 * nq + 16 * M + 32 * Mc}
    kernels = {}
    for k, b_ in stage_bytes.items():
        if k not in bd:
            continue
        gbs = b_ / (bd[k] * 1e-6) / 1e9
        kernels[k] = {"algorithmic_bytes": b_, "us": bd[k], "achieved": gbs, "frac": gbs / peak,
                      "traffic": traffic.get(k)}
    if fused_paint and "paint" in kernels:
        kernels["paint"]["note"] = ("timed standalone (k_paint); in the step the deposits are "
                                    "made by the rRESPA launch")

    ns_day = sps * cfg.respa_inner * cfg.time_step * 86400 / 1000.0
    # CPU baseline (rank 0, N=1 only): bounded oracle sample
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        c_sps, c_secs, c_done, c_thr = cpu_baseline(s, steps=3, budget_s=30.0)
        cpu = {"value": c_sps, "unit": "steps/s", "cores": c_thr, "kind": "port",
               "sample": f"{c_done} outer steps of the full workload ({c_secs:.1f} s) on the "
                         "FP32 restatement of the reference's step (oracle/cpu_md.py), OpenMP "
                         f"over {c_thr} threads and FFTs over {os.cpu_count()} workers"}
    if rank == 0:
        info = md.plan_info() or {}
        # one warp per molecule group up to 64 beads, one CTA per group beyond
        warp = max(md.block_beads or 0, info.get("max_block_beads", 0)) <= 64
        respa_kernel = "k_respa_warp" if warp else "k_respa_cta"
        line = {"metric": METRIC, "value": sps * ws, "unit": "steps/s", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 (f64 energies/virial)", "data": "synthetic",
                "ns_per_day": ns_day * ws,
                "config": _config_block(cfg, n, args.workload),
                "gpu_setup": {"bead_order": "sorted by mesh cell at setup",
                              "paint": ("fused into the rRESPA launch (free beads in a "
                                        "kernel of their own beside the molecule groups)"
                                        if fused_paint else "separate launch"),
                              "charge_chain": ("second stream beside the density chain"
                                               if md.charges is not None else None),
                              "respa_groups": md.plan_info(),
                              "respa_group_tuning_us": md.block_timings,
                              "kspace_tile": md.pm.spectral_tile,
                              "kspace_tile_tuning_us": md.spectral_tile_timings},
                "e2e": {"value": e2e_sps * ws, "unit": "steps/s",
                        "h2d_bytes_per_step": e2e_h2d, "d2h_bytes_per_step": e2e_d2h,
                        "transfer": "RespaMD.run_host (r, v in; r out; page-locked host "
                                    "memory), host wall clock around the call + synchronize"},
                "e2e_dropin": dropin,
                "after_1000_steps": aged,
                "accuracy": acc,
                "gpu_launches": md.launches_per_step * args.steps,
                "roofline": {"kernel": f"{respa_kernel} (fused rRESPA inner loop, "
                                       f"{cfg.respa_inner} inner steps per launch)",
                             "bound": "hbm", "achieved": respa_gbs, "peak": peak, "unit": "GB/s",
                             "frac": respa_gbs / peak, "traffic": traffic.get("respa"),
                             "peak_kind": peak_kind, "ms_per_launch": respa_ms,
                             "algorithmic_bytes": respa_bytes,
                             "bytes_basis": "respa_inner x (72 N + 16 B + 20 A + 144 D), "
                                            "the unfused inner step's reads and writes"
                                            + (", + the fused paint's 16 N + 4 T M (+ 16 N_q "
                                               "+ 4 M for the charges)" if fused_paint else ""),
                             "note": "latency-bound in practice: the loop runs on chip and "
                                     "touches DRAM once per bead per launch (traffic)"},
                "roofline_kernels": kernels,
                "adjoint": adj,
                "clocks": clk.summary(),
                "cpu_baseline": cpu}
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_replicas(args):
    """64 independent replicas (melt and membrane recipes, 5k-200k beads,
    meshes 32^3-64^3, chi uniform in [5, 40]) advanced as one captured graph
    per step, against the same replicas stepped one by one (each replica's
    own step graph, replayed in turn).  value = replica-steps/s."""
    import torch
    from hymd_gb300 import systems
    from hymd_gb300.replicas import ReplicaBatch
    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    sys_ = systems.replica_set(n_replicas=64, seed=5 + rank)
    rb = ReplicaBatch(sys_, device=dev, seed=100 + rank)
    rb.prime()
    rb.measure_each()
    flush = L2Flush(torch, dev)
    st = torch.cuda.current_stream()

    def timed(step_fn):
        for _ in range(max(3, args.warmup)):
            step_fn()
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        for a, b in evs:
            flush.zero_()
            a.record(st)
            step_fn()
            b.record(st)
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in evs) / args.steps

    seq_ms = max_over_ranks(timed(lambda: rb.run_sequential(1)), ws, dev)
    k = rb.tune_streams()
    with ClockSampler(local) as clk:
        bat_ms = max_over_ranks(timed(lambda: rb.run(1)), ws, dev)
    rb.check_errors()
    R = len(rb.replicas)
    line = {"metric": "aggregate replica MD steps/s (64 replicas, one graph per step)",
            "value": R * 1000.0 / bat_ms * ws, "unit": "replica-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": bat_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (f64 energies/virial)", "data": "synthetic",
            "replica_by_replica": {"value": R * 1000.0 / seq_ms * ws, "ms_per_step": seq_ms},
            "speedup_vs_replica_by_replica": seq_ms / bat_ms,
            "config": {"workload": "64 replicas: melt and membrane recipes, beads log-uniform "
                                   "5k-200k at 8.3 nm^-3, mesh 32^3-64^3 at ~0.4 nm, chi "
                                   "uniform [5, 40], CSVR 323 K",
                       "n_beads_total": int(sum(rb.n_beads)), "streams": rb.n_streams,
                       "stream_tuning_ms": {str(k): v / 1000.0
                                            for k, v in (rb.stream_timings or {}).items()},
                       "l2": "flushed between timed steps", "parallelism": "replicas only"},
            "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line))
    return 0


def run_topology(args):
    """prepare_bonds (hymd/force.py:325-505 + 573-728) on the device for the
    1.3M-bead membrane (108k lipids + W, every bead its own molecule id when
    free): wall time per call, inputs on the host and the packed arrays back
    on the host as the reference returns them, checked against the tiled
    per-molecule result.  Beside it, the host restatement (the reference's
    traversals in Python without networkx) on the 162k-bead membrane."""
    import time
    import torch
    from hymd_gb300 import systems
    from hymd_gb300.force import prepare_bonds
    ws, rank = _dist()
    if rank != 0:
        return 0
    torch.cuda.set_device(0)
    n_total = 1_300_000
    n_lipids = int(round(0.444 * n_total / 12))
    s = systems.lipid_membrane(seed=7, n_lipids=n_lipids, n_water=n_total - 12 * n_lipids,
                               box=54.0, mesh=128)
    n = len(s["names"])
    idx = np.arange(n)
    call = lambda: prepare_bonds(s["molecules"], s["names"], s["bonds"], idx, s["config"],
                                 device="cuda")
    for _ in range(max(args.warmup, 1)):
        packed = call()
    assert all(x.dtype == y.dtype and np.array_equal(x, y) for x, y in zip(packed, s["topology"]))
    times = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        call()
        times.append(time.perf_counter() - t0)
    dev_s = float(np.median(times))
    m = systems.lipid_membrane()
    t0 = time.perf_counter()
    host = prepare_bonds(m["molecules"], m["names"], m["bonds"], np.arange(len(m["names"])),
                         m["config"])
    host_s = time.perf_counter() - t0
    assert all(np.array_equal(x, y) for x, y in zip(host, m["topology"]))
    line = {"metric": "bonded-term discovery time (prepare_bonds), 1.3M-bead membrane",
            "value": dev_s, "unit": "s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(args.warmup, 1), "higher_is_better": False, "vs_baseline": None,
            "dtype": "int32", "data": "synthetic",
            "terms": {"bonds": len(packed[0]), "angles": len(packed[4]),
                      "dihedrals": len(packed[9])},
            "host_restatement": {"value": host_s, "unit": "s", "cores": 1,
                                 "sample": f"162k-bead membrane ({len(m['names'])} beads, "
                                           "6000 lipids), Python traversal"},
            "config": {"workload": f"lipid membrane {n} beads ({n_lipids} lipids + W), "
                                   "box 54 nm", "timed": "host inputs -> packed host arrays"}}
    print(json.dumps(line))
    return 0


def run_gpe(args):
    """PIC_Spectral_GPE electrostatics (hymd/field.py:764-1112) through the
    drop-in update_field_force_q_GPE on the charged-peptide recipe (500k
    beads, box 40 nm, mesh 128^3; dielectric 2 / 10 / 80 for BB / SC / W,
    max_diff convergence to 1e-6, mixing 0.6): wall time per solve with the
    filtered densities already on the device, the iteration count, and the
    FP64 oracle's solve of the same system on one host core beside it, with
    the forces, energy and iterations compared."""
    import time
    import torch
    from hymd_gb300 import field as gf, systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from oracle import field as of
    from oracle import hamiltonian as oh
    ws, rank = _dist()
    if rank != 0:
        return 0
    torch.cuda.set_device(0)
    s = systems.charged_peptides(seed=2)
    cfg = s["config"]
    cfg.coulombtype = "PIC_Spectral_GPE"
    cfg.dielectric_type = [2.0, 10.0, 80.0]
    cfg.conv_crit, cfg.pol_mixing, cfg.convergence_type = 1e-6, 0.6, "max_diff"
    T = cfg.n_types
    ham = get_hamiltonian(cfg)
    pm, fl, ecl, cl = gf.initialize_pm(None, cfg)
    phi, phi_fourier, force_on_grid, v_ext_fourier, v_ext, phi_transfer, phi_lap = fl
    phi_q, phi_q_fourier, psi, elec_field = ecl
    (phi_eps, phi_eps_fourier, phi_eta, phi_eta_fourier, phi_pol, phi_pol_prev, elec_dot,
     elec_field_contrib, Vbar_elec, Vbar_elec_fourier, force_mesh_elec,
     force_mesh_elec_fourier) = cl
    R = torch.as_tensor(s["positions"], device="cuda")
    Ty = torch.as_tensor(s["types"], device="cuda")
    Q = torch.as_tensor(s["charges"], device="cuda")
    gf.update_field(phi, phi_lap, phi_transfer, None, force_on_grid, ham, pm, R, Ty, cfg, v_ext,
                    phi_fourier, v_ext_fourier, cfg.m)
    F = torch.zeros_like(R)

    def solve():
        out = gf.update_field_force_q_GPE(
            None, phi, Ty, Q, phi_q, phi_q_fourier, phi_eps, phi_eps_fourier, phi_eta,
            phi_eta_fourier, phi_pol_prev, phi_pol, elec_field, F, elec_field_contrib, psi,
            Vbar_elec, Vbar_elec_fourier, force_mesh_elec, force_mesh_elec_fourier, ham, None,
            None, pm, R, cfg)
        torch.cuda.synchronize()
        return out

    for _ in range(max(args.warmup, 1)):
        solve()
    times = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, eps_g, dot = solve()
        times.append(time.perf_counter() - t0)
    dev_ms = 1000.0 * float(np.median(times))
    iters = int(pm.gpe_iterations)
    W = gf.compute_field_energy_q_GPE(cfg, eps_g, None, dot)
    line = {"metric": "PIC_Spectral_GPE solve time (update_field_force_q_GPE)",
            "value": dev_ms, "unit": "ms", "n_gpus": 1, "steps": args.steps,
            "warmup": max(args.warmup, 1), "higher_is_better": False, "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "iterations": iters,
            "ms_per_iteration": dev_ms / max(iters, 1),
            "config": {"workload": "charged peptides 500k beads, box 40 nm, mesh 128^3, "
                                   "3 types, dielectric 2/10/80",
                       "timed": "wall time of one solve (densities resident), host "
                                "synchronisations included"}}
    if args.no_cpu_baseline:
        print(json.dumps(line))
        return 0
    # the FP64 oracle on the same inputs: filtered densities, then the solve
    names = cfg.unique_names
    chim = np.zeros((T, T))
    for c in cfg.chi:
        i, j = names.index(c.atom_1), names.index(c.atom_2)
        chim[i, j] = chim[j, i] = c.interaction_energy
    fun = oh.quadratic_from_params("DefaultWithChi", T, cfg.kappa, cfg.rho0, cfg.a, chim)
    r64 = s["positions"].astype(np.float64)
    ref_field = of.update_field(r64, s["types"], T, cfg.mesh(), cfg.box(), cfg.m, fun, cfg.sigma)
    nshape = tuple(cfg.mesh())
    state = dict(phi_eps=np.zeros(nshape), pol_prev=np.zeros(nshape), contrib=np.zeros(nshape))
    t0 = time.perf_counter()
    ref = of.gpe_step(ref_field["phi"], s["charges"], s["positions"], s["types"], T, cfg.mesh(),
                      cfg.box(), cfg.sigma, cfg.dielectric_type, cfg.type_charges or [0.0] * T,
                      state, conv_crit=cfg.conv_crit, mixing=cfg.pol_mixing, conv_kind="max_diff")
    cpu_s = time.perf_counter() - t0
    f_ref = ref["forces"]
    f_rel = float(np.sqrt(np.mean((F.cpu().numpy() - f_ref) ** 2)) / np.sqrt(np.mean(f_ref ** 2)))
    line["accuracy"] = {"reference": "FP64 oracle (oracle/field.py:gpe_step) on the same "
                                     "inputs", "force_rel_rms": f_rel,
                        "energy_rel_err": abs(W - ref["energy"]) / abs(ref["energy"]),
                        "oracle_iterations": int(ref["iterations"])}
    line["cpu_baseline"] = {"value": 1000.0 * cpu_s, "unit": "ms", "cores": 1, "kind": "port",
                            "sample": "the whole solve, FP64 numpy oracle"}
    print(json.dumps(line))
    return 0


def run_trajectory(args):
    """Trajectory and observable output (hymd/file_io.py:527-779 through
    TrajectoryRecorder) on the default MD workload (500k charged peptides,
    mesh 128^3): steps/s of the captured step replayed K times without
    output, then with a frame every n_print = 10 steps (positions,
    velocities and total forces in the caller's bead order, FP64 field and
    electrostatic energies, pressure) copied to page-locked host memory on a
    side stream and written to an in-memory H5MD tree while the next steps
    run.  Host wall clock around the whole run, the last frame written."""
    import tempfile
    import time
    import torch
    from hymd_gb300 import file_io as fio
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    from hymd_gb300.trajectory import TrajectoryRecorder
    ws, rank = _dist()
    if rank != 0:
        return 0
    torch.cuda.set_device(0)
    K, n_print = max(args.steps, 10), 10
    s = systems.charged_peptides(seed=2)
    cfg = s["config"]
    cfg.n_steps, cfg.n_print = K, n_print
    ham = get_hamiltonian(cfg)
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham, topology=s["topology"],
                 charges=s["charges"])
    md.sort_particles()
    md.couple(thermostat=True, seed=100, n_steps=2 * K + args.warmup + 8)
    md.prime()
    md.capture()
    md.run(max(args.warmup, 3))
    torch.cuda.synchronize()

    def timed(with_output):
        rec = None
        if with_output:
            out = fio.OutDataset(tempfile.mkdtemp(), cfg, backend="memory")
            topo = s["topology"]
            fio.store_static(out, list(range(md.n)), s["names"], s["types"], np.arange(md.n),
                             cfg, topo[0], topo[1], molecules=s["molecules"], velocity_out=True,
                             force_out=True, charges=s["charges"])
            rec = TrajectoryRecorder(md, out, ham, velocity_out=True, force_out=True,
                                     pressure=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for step in range(1, K + 1):
            md.run(1)
            if rec is not None and step % n_print == 0:
                rec.record(step)
                rec.drain()
        if rec is not None:
            rec.close()
        torch.cuda.synchronize()
        return time.perf_counter() - t0, (rec.written if rec is not None else 0)

    t_plain, _ = timed(False)
    t_out, frames = timed(True)
    line = {"metric": "MD steps/s with trajectory output every n_print steps",
            "value": K / t_out, "unit": "steps/s", "n_gpus": 1, "steps": K,
            "warmup": max(args.warmup, 3), "higher_is_better": True, "vs_baseline": None,
            "dtype": "f32 (f64 energies)", "data": "synthetic",
            "without_output": K / t_plain, "frames": frames, "n_print": n_print,
            "ms_per_frame_overhead": 1000.0 * (t_out - t_plain) / max(frames, 1),
            "frame_bytes_d2h": int(3 * 12 * md.n + 2 * 32 * 8),
            "config": {"workload": WORKLOADS["peptide500k"][0],
                       "output": "positions, velocities, forces (caller order), energies, "
                                 "pressure; in-memory H5MD tree",
                       "timed": "host wall clock over the K steps, output drained and closed"}}
    print(json.dumps(line))
    return 0


def run_plumed(args):
    """The PLUMED bias coupling (hymd/plumed.py:11-235 through PlumedBias and
    RespaMD.set_bias) on the default MD workload (500k charged peptides):
    steps/s with a bias evaluated after every field step (a DISTANCE
    restraint between two beads of the first chain, as the reference's PLUMED
    test input) against the same steps without it.  py-plumed is not
    installed: the PLUMED kernel is the stand-in of the tests
    (tests/plumed_fake.py), so the time is this package's coupling: the
    positions and forces copied to the host every step, the bias force copied
    back into the outer kicks, and eager launches (a biased run is not
    captured in a graph)."""
    import tempfile
    import time
    import torch
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    from hymd_gb300.plumed import PlumedBias
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests"))
    from plumed_fake import FakePlumed
    ws, rank = _dist()
    if rank != 0:
        return 0
    torch.cuda.set_device(0)
    K = max(args.steps, 10)
    s = systems.charged_peptides(seed=2)
    cfg = s["config"]
    ham = get_hamiltonian(cfg)

    def make(bias):
        md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, ham,
                     topology=s["topology"], charges=s["charges"])
        md.couple(thermostat=True, seed=100, n_steps=K + args.warmup + 8)
        if bias:
            d = tempfile.mkdtemp()
            dat = os.path.join(d, "plumed.dat")
            with open(dat, "w") as f:
                f.write("d: DISTANCE ATOMS=3,17\nRESTRAINT ARG=d KAPPA=4000.0 AT=0.8\n")
            md.set_bias(PlumedBias(cfg, dat, os.path.join(d, "log"), kernel=FakePlumed()))
        md.prime()
        return md

    def timed(md):
        for _ in range(max(args.warmup, 3)):
            md.step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(K):
            md.step()
        torch.cuda.synchronize()
        return K / (time.perf_counter() - t0)

    plain = timed(make(False))
    biased = timed(make(True))
    line = {"metric": "MD steps/s with a PLUMED bias every step", "value": biased,
            "unit": "steps/s", "n_gpus": 1, "steps": K, "warmup": max(args.warmup, 3),
            "higher_is_better": True, "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "without_bias_eager": plain, "ms_per_step_overhead": 1000.0 * (1.0 / biased - 1.0 / plain),
            "config": {"workload": WORKLOADS["peptide500k"][0],
                       "bias": "DISTANCE of beads 3 and 17 + RESTRAINT (stand-in PLUMED kernel)",
                       "timed": "host wall clock, eager steps (a bias runs on the host)"}}
    print(json.dumps(line))
    return 0


def run_reverse(args):
    """Reverse mode on the membrane recipe scaled to 1.3M beads (54 nm box,
    mesh 128^3): the gradient with respect to chi of the MSE between the
    z-density profile (100 bins per type) averaged over K outer steps and a
    target made by the same K-step run with chi perturbed by seeded N(0, 1)
    kJ/mol; sqrt(K) checkpoints.  Also the adjoint's cost on this system."""
    import torch
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    from hymd_gb300.reverse import ForceModel, profile_loss
    ws, rank = _dist()
    if rank != 0:
        return 0
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    n_total, box = 1_300_000, 54.0
    n_lipids = int(round(0.444 * n_total / 12))
    s = systems.lipid_membrane(seed=7, n_lipids=n_lipids, n_water=n_total - 12 * n_lipids,
                               box=box, mesh=128)
    cfg = s["config"]
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, get_hamiltonian(cfg),
                 topology=s["topology"], device=dev)
    model = ForceModel(md)
    T = cfg.n_types
    names = cfg.unique_names
    chi0 = np.zeros((T, T))
    for c in cfg.chi:
        i, j = names.index(c.atom_1), names.index(c.atom_2)
        chi0[i, j] = chi0[j, i] = c.interaction_energy
    rng = np.random.default_rng(17)
    pert = np.triu(rng.normal(0.0, 1.0, (T, T)), 1)
    chi_target = chi0 + pert + pert.T
    K, n_bins = args.reverse_steps, 100
    x0, v0 = md.r.clone(), md.v.clone()
    zero = torch.zeros((T, n_bins), dtype=torch.float32, device=dev)
    with torch.no_grad():
        _, target = profile_loss(x0, v0, torch.tensor(chi_target, dtype=torch.float32,
                                                      device=dev), model, K, zero, n_bins)
    chi = torch.tensor(chi0, dtype=torch.float32, device=dev, requires_grad=True)
    # one untimed pass of each (the allocator's first growth, cuFFT plans)
    with torch.no_grad():
        profile_loss(x0, v0, chi.detach(), model, K, target, n_bins)
    warm, _ = profile_loss(x0, v0, chi, model, K, target, n_bins)
    warm.backward()
    chi.grad = None
    torch.cuda.synchronize()
    a, b, c = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    with torch.no_grad():
        a.record()
        profile_loss(x0, v0, chi.detach(), model, K, target, n_bins)
        b.record()
    b.synchronize()
    fwd_ms = a.elapsed_time(b)
    torch.cuda.reset_peak_memory_stats(dev)
    a.record()
    loss, _ = profile_loss(x0, v0, chi, model, K, target, n_bins)
    loss.backward()
    c.record()
    c.synchronize()
    fb_ms = a.elapsed_time(c)
    peak_gb = torch.cuda.max_memory_allocated(dev) / 1e9
    g = chi.grad.detach().cpu().numpy()
    flush = L2Flush(torch, dev)
    adj = adjoint_cost(md, flush, torch)
    # the MD force against the exact derivative of the discrete field energy
    # on three meshes of the same configuration
    from hymd_gb300 import adjoint
    from hymd_gb300.field import ParticleMesh
    gaps = {}
    for nm in (64, 128, 256):
        pm = ParticleMesh([nm] * 3, cfg.box(), T, device=dev)
        gaps[str(nm)] = adjoint.gradient_gap(x0, md.types, pm, cfg.m, chi0, cfg.kappa, cfg.sigma,
                                             cfg.rho0, cfg.a if cfg.a is not None else cfg.rho0)
        del pm
    torch.cuda.empty_cache()
    pep = reverse_peptides(dev, K=min(K, 50))
    line = {"metric": "reverse-mode K-step gradient of a z-profile loss w.r.t. chi (s)",
            "value": fb_ms / 1000.0, "unit": "s", "n_gpus": 1, "steps": K, "warmup": 0,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (f64 energies)", "data": "synthetic",
            "forward_only_s": fwd_ms / 1000.0, "backward_over_forward": fb_ms / fwd_ms - 1.0,
            "peak_device_memory_gb": peak_gb, "loss": float(loss.detach()),
            "grad_chi_pairs": {f"{names[i]}-{names[j]}": float(g[i, j] + g[j, i])
                               for i in range(T) for j in range(i + 1, T)},
            "adjoint": adj,
            "gradient_gap_by_mesh": {"value": gaps, "unit": "||F + dW/dx|| / ||F||",
                                     "box_nm": box},
            "peptides_dihedrals_csvr": pep,
            "config": {"workload": f"lipid membrane {md.n} beads ({n_lipids} lipids + W), "
                                   f"box {box} nm, mesh 128^3, 5 types",
                       "K": K, "checkpoint_every": int(np.ceil(np.sqrt(K))),
                       "respa_inner": int(cfg.respa_inner), "ensemble": "NVE",
                       "target": "same K-step run with chi + seeded N(0,1) kJ/mol"}}
    print(json.dumps(line))
    return 0


def reverse_peptides(dev, K=50):
    """The reverse-mode gradient on the charged peptide recipe (500k beads:
    200 chains of 50 residues with CBT four-body terms, side-chain and
    counter-ion charges under PIC_Spectral, mesh 128^3) in NVT (CSVR every
    outer step): forward and forward + backward times after one untimed
    pass of each."""
    import torch
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    from hymd_gb300.reverse import ForceModel, profile_loss
    s = systems.charged_peptides(seed=2)
    cfg = s["config"]
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, get_hamiltonian(cfg),
                 topology=s["topology"], device=dev, charges=s["charges"])
    md.couple(thermostat=True, seed=11, n_steps=max(K, 1) + 1)
    model = ForceModel(md)
    T = cfg.n_types
    names = cfg.unique_names
    chi0 = np.zeros((T, T))
    for c in cfg.chi:
        i, j = names.index(c.atom_1), names.index(c.atom_2)
        chi0[i, j] = chi0[j, i] = c.interaction_energy
    n_bins = 100
    x0, v0 = md.r.clone(), md.v.clone()
    target = torch.zeros((T, n_bins), dtype=torch.float32, device=dev)
    chi = torch.tensor(chi0, dtype=torch.float32, device=dev, requires_grad=True)
    with torch.no_grad():
        profile_loss(x0, v0, chi.detach(), model, K, target, n_bins)
    warm, _ = profile_loss(x0, v0, chi, model, K, target, n_bins)
    warm.backward()
    chi.grad = None
    a, b, c = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    torch.cuda.synchronize()
    with torch.no_grad():
        a.record()
        profile_loss(x0, v0, chi.detach(), model, K, target, n_bins)
        b.record()
    b.synchronize()
    fwd_ms = a.elapsed_time(b)
    a.record()
    loss, _ = profile_loss(x0, v0, chi, model, K, target, n_bins)
    loss.backward()
    c.record()
    c.synchronize()
    fb_ms = a.elapsed_time(c)
    out = {"n_beads": md.n, "K": K, "dihedrals": md.topo.n_dihedrals,
           "ensemble": "NVT (CSVR)", "forward_only_s": fwd_ms / 1000.0,
           "forward_backward_s": fb_ms / 1000.0, "backward_over_forward": fb_ms / fwd_ms - 1.0,
           "charged_beads": int(np.count_nonzero(s["charges"]))}
    del md, model
    torch.cuda.empty_cache()
    return out


def run_locality(args):
    """Step time (graph replays, CUDA events, L2 flushed before each) against
    the age of the bead order, for both mesh-cell sort orders: right after
    the sort, then after more and more unsorted steps; then the device time
    of resort() (the first one records its graph) and the step time right
    after the re-sorts.  Diagnostic; prints one JSON object per order."""
    import torch
    from hymd_gb300 import systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    s = systems.BUILDERS[args.workload](seed=2)
    cfg = s["config"]
    flush = L2Flush(torch, dev)
    st = torch.cuda.current_stream()
    for order in ("molecule", "bead"):
        md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, get_hamiltonian(cfg),
                     topology=s["topology"], charges=s.get("charges"), device=dev)
        md.sort_particles(order=order)
        md.couple(seed=100, n_steps=20000, **WORKLOADS[args.workload][1])
        md.prime()
        md.capture()

        def timed(k=20):
            tot = 0.0
            for _ in range(k):
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(st)
                md.replay()
                b.record(st)
                b.synchronize()
                tot += a.elapsed_time(b)
            return round(1000.0 * tot / k, 1)

        ages = {}
        md.run(3)
        age = 3
        for target in (3, 50, 200, 1000, 3000):
            md.run(target - age)
            age = target
            ages[str(age)] = timed()
            age += 20
        resort = []
        for _ in range(5):
            flush.zero_()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            md.resort()
            b.record(st)
            b.synchronize()
            resort.append(round(1000.0 * a.elapsed_time(b), 1))
        after = timed()
        md.check_errors()
        print(json.dumps({"workload": args.workload, "order": order, "step_us_by_age": ages,
                          "step_us_after_resort": after, "resort_us": resort}))
        del md
        torch.cuda.empty_cache()
    return 0


def profile_stage(args):
    """Run one stage of the step eagerly (no graph, no timing) `--reps` times
    on the workload and exit: a small program for kernel profilers.
    Stages: paint, field (paint -> r2c -> k-space -> c2r -> readout), respa
    (the fused inner loop), step (a whole outer step)."""
    import torch
    from hymd_gb300 import _lib, systems
    from hymd_gb300.hamiltonian import get_hamiltonian
    from hymd_gb300.md import RespaMD

    s = systems.BUILDERS[args.workload](seed=2)
    cfg = s["config"]
    md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, get_hamiltonian(cfg),
                 topology=s["topology"], charges=s.get("charges"))
    md.sort_particles()
    md.couple(seed=100, n_steps=max(16, 4 * args.reps), **WORKLOADS[args.workload][1])
    md.prime()
    phi = md.pm.real_field(cfg.n_types)
    masses = _lib.dvec(cfg.m)
    st = _lib.stream_ptr()
    for _ in range(args.reps):
        if args.profile_stage == "paint":
            _lib.call("hpf_paint", md.pm._h, _lib.ptr(md.r), _lib.ptr(md.types), md.n, masses,
                      _lib.ptr(phi), st)
        elif args.profile_stage == "field":
            md._field(st, md.field_sums)
        elif args.profile_stage == "respa":
            md._inner_fused(st)
        else:
            md.step()
    torch.cuda.synchronize()
    md.check_errors()
    print(json.dumps({"profile_stage": args.profile_stage, "workload": args.workload,
                      "reps": args.reps, "status": "ok"}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="hpf", choices=["hpf", "reference"])
    ap.add_argument("--workload", default=WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the FP64-oracle accuracy check of the timed state")
    ap.add_argument("--no-aging", action="store_true",
                    help="skip the second timing after 1000 further steps")
    ap.add_argument("--no-dropin", action="store_true",
                    help="skip the drop-in-API end-to-end measurement")
    ap.add_argument("--breakdown", action="store_true",
                    help="also print per-phase step times (us) to stderr")
    ap.add_argument("--profile-stage", choices=["paint", "field", "respa", "step"],
                    help="run one stage eagerly --reps times for a profiler, print no bench line")
    ap.add_argument("--reps", type=int, default=4)
    ap.add_argument("--replicas", action="store_true",
                    help="batched 64-replica workload instead of a single system")
    ap.add_argument("--reverse", action="store_true",
                    help="reverse-mode chi gradient on the 1.3M-bead membrane")
    ap.add_argument("--reverse-steps", type=int, default=200)
    ap.add_argument("--locality", action="store_true",
                    help="diagnostic: step time against the age of the bead order")
    ap.add_argument("--plumed", action="store_true",
                    help="MD steps/s with a PLUMED bias every step (one JSON line)")
    ap.add_argument("--trajectory", action="store_true",
                    help="MD steps/s with trajectory output every 10 steps (one JSON line)")
    ap.add_argument("--gpe", action="store_true",
                    help="PIC_Spectral_GPE solve time on the 500k peptides (one JSON line)")
    ap.add_argument("--topology", action="store_true",
                    help="bonded-term discovery (prepare_bonds) on the device, 1.3M-bead membrane")
    args = ap.parse_args()
    if args.profile_stage:
        return profile_stage(args)
    if args.replicas:
        return run_replicas(args)
    if args.reverse:
        return run_reverse(args)
    if args.topology:
        return run_topology(args)
    if args.gpe:
        return run_gpe(args)
    if args.trajectory:
        return run_trajectory(args)
    if args.plumed:
        return run_plumed(args)
    if args.locality:
        return run_locality(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
