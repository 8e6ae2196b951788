"""Many independent hPF-MD replicas advanced together on one GPU.

Each replica is a full `RespaMD` (its own mesh context, cuFFT plans, rRESPA
plan and coupling state); the replicas differ in chi, particle count and
mesh size.  One outer step of ALL replicas is captured as a single CUDA
graph: the capture stream forks into `n_streams` side streams, each side
stream records the step sequences of its share of the replicas, and the
branches join again, so that a replay is one graph launch per step whose
independent branches run concurrently and fill the GPU that one small
replica leaves mostly idle.  Replicas are assigned to streams by
longest-processing-time first on their measured single-replica step times,
and the number of streams is picked by timing the candidates
(`tune_streams`).

The replica-by-replica form (`run_sequential`) replays each replica's own
step graph one after another: the same kernels, without the concurrency.
"""
import numpy as np
import torch

from .hamiltonian import get_hamiltonian
from .md import RespaMD


class ReplicaBatch:
    def __init__(self, systems, device="cuda", thermostat=True, seed=0, n_steps=100000,
                 sort=True):
        self.device = torch.device(device)
        self.replicas = []
        for i, s in enumerate(systems):
            cfg = s["config"]
            md = RespaMD(s["positions"], s["velocities"], s["types"], cfg, get_hamiltonian(cfg),
                         topology=s.get("topology"), charges=s.get("charges"), device=self.device)
            if sort:
                md.sort_particles()
            md.couple(thermostat=thermostat, barostat=None, seed=seed + i, n_steps=n_steps)
            self.replicas.append(md)
        self.n_beads = [md.n for md in self.replicas]
        self.graph = None
        self.step_us = None
        self.n_streams = None
        self.stream_timings = None

    def prime(self):
        for md in self.replicas:
            md.prime()
        torch.cuda.synchronize(self.device)

    # ------------------------------------------------------------------
    def capture_each(self):
        """Per-replica step graphs (the replica-by-replica form)."""
        for md in self.replicas:
            if md.graph is None:
                md.capture()

    def run_sequential(self, steps=1):
        for _ in range(steps):
            for md in self.replicas:
                md.graph.replay()

    def measure_each(self, reps=5):
        """Device time (us) of one step of each replica alone (graph replay)."""
        self.capture_each()
        st = torch.cuda.current_stream(self.device)
        out = []
        for md in self.replicas:
            md.graph.replay()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            for _ in range(reps):
                md.graph.replay()
            b.record(st)
            b.synchronize()
            out.append(a.elapsed_time(b) * 1000.0 / reps)
        self.step_us = out
        return out

    def _assign(self, n_streams):
        cost = self.step_us if self.step_us is not None else [float(n) for n in self.n_beads]
        order = np.argsort(cost)[::-1]
        load = np.zeros(n_streams)
        groups = [[] for _ in range(n_streams)]
        for i in order:
            k = int(np.argmin(load))
            groups[k].append(int(i))
            load[k] += cost[i]
        return [g for g in groups if g]

    def capture(self, n_streams=8):
        """One CUDA graph for one outer step of every replica, with the
        replicas spread over `n_streams` concurrent branches."""
        groups = self._assign(n_streams)
        cur = torch.cuda.current_stream(self.device)
        streams = [torch.cuda.Stream(device=self.device) for _ in groups]
        # warm-up on the side streams (first use of every code path)
        for s, grp in zip(streams, groups):
            s.wait_stream(cur)
            with torch.cuda.stream(s):
                for i in grp:
                    self.replicas[i].step()
        for s in streams:
            cur.wait_stream(s)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            cap = torch.cuda.current_stream(self.device)
            for s, grp in zip(streams, groups):
                s.wait_stream(cap)
                with torch.cuda.stream(s):
                    for i in grp:
                        self.replicas[i].step()
            for s in streams:
                cap.wait_stream(s)
        self.graph = g
        self.n_streams = len(groups)
        self._streams = streams
        return g

    def run(self, steps=1):
        for _ in range(steps):
            self.graph.replay()

    def tune_streams(self, candidates=(4, 8, 16, 32), reps=3):
        """Capture the batched step with each stream count, time it, keep the
        fastest (timings in `stream_timings`, us per batched step)."""
        if self.step_us is None:
            self.measure_each()
        st = torch.cuda.current_stream(self.device)
        best, timings = None, {}
        for k in candidates:
            if k > len(self.replicas):
                continue
            self.capture(k)
            self.graph.replay()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            for _ in range(reps):
                self.graph.replay()
            b.record(st)
            b.synchronize()
            t = a.elapsed_time(b) * 1000.0 / reps
            timings[k] = t
            if best is None or t < best[0]:
                best = (t, k)
        self.stream_timings = timings
        self.capture(best[1])
        return best[1]

    def check_errors(self):
        for md in self.replicas:
            md.check_errors()
