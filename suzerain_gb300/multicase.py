"""Many independent cases of uneven size advanced together (configuration 3).

Each case (S, Ny, k and its own wavenumber grid) is one resident ``Plan``:
its bands, coefficients, factors and refinement state stay on the device.
A step advances every case through the SMR91 substeps.  The cases are spread
over several CUDA streams so that small cases fill the SMs that a large case
leaves idle, and the whole step (every case, every substep) is recorded once
into a CUDA graph and replayed: one graph launch per step, no host
synchronization inside it (the plans run their capturable substep, whose
refinement loops are bounded by device-side counts).

The factor shape of every distinct geometry (N, KL, KU) is chosen by the
tuner before capture, on that geometry's own cases.

Ragged mode (``ragged=True``) factors every case's systems of a substep in
one launch per row-tile class instead of one launch per case:
each case runs stage 1 of its substep (explicit operator, refinement
initial state) on its stream, one ragged factor runs over all cases, and
each case runs stage 2 (solves, refinement, fallback) on its stream again.
The results are those of the per-case form bit for bit.
"""
from __future__ import annotations

import numpy as np

from . import plan as P
from . import synth
from . import tune as T


class MultiCase:
    def __init__(self, configs: list, nstreams: int = 8, max_double_slots: int = 128,
                 complex_coupling: bool = False, ragged: bool = False):
        import torch
        self.torch = torch
        self.ragged = bool(ragged)
        self.ragged_factors = {}     # substep -> RaggedFactor (built at capture)
        self.configs = list(configs)
        self.nstreams = max(1, int(nstreams))
        self.cases, self.plans, self.u0, self.bufs = [], [], [], []
        for c in self.configs:
            cs, kx, kz, u = c.batch(complex_coupling)
            synth.zero_dirichlet_rows(cs, u)
            self.cases.append(cs)
            self.plans.append(P.Plan(cs, kx, kz, max_double_slots=min(max_double_slots, len(kx))))
            du = torch.from_numpy(u).cuda()
            self.u0.append(du)
            # ping-pong state buffers: substep i reads bufs[i % 2], writes the other
            self.bufs.append([du.clone(), torch.empty_like(du)])
        self.streams = [torch.cuda.Stream() for _ in range(self.nstreams)]
        self.graph = None
        self.nsubsteps = 0

    @property
    def nsys(self) -> int:
        return sum(p.nsys for p in self.plans)

    def device_bytes(self) -> int:
        return sum(p.device_bytes() for p in self.plans) + sum(
            2 * b[0].numel() * b[0].element_size() for b in self.bufs)

    def geometries(self) -> dict:
        """{(N, KL, KU): [case indices]}"""
        g = {}
        for i, cs in enumerate(self.cases):
            g.setdefault((cs.N, cs.KL, cs.KU), []).append(i)
        return g

    def tune(self, precs: str = "C", nsys: int = 512, reps: int = 2) -> dict:
        """Time the factor shapes once per distinct geometry (packed band of
        that geometry, up to nsys systems) and record the fastest."""
        out = {}
        for (N, KL, KU), idx in self.geometries().items():
            n = min(nsys, max(self.plans[i].nsys for i in idx))
            for prec in precs:
                out[(prec, N, KL, KU)] = T.tune_packed(prec, N, KL, KU, nsys=n, reps=reps)["best"]
        return out

    def _phis(self, ci: int, i: int):
        c = self.configs[ci]
        return synth.smr91_phis(c.phi * synth.SMR91_BETA[i] / synth.SMR91_BETA[0], substep=i)

    def _ragged_factor(self, i: int, spec):
        """The ragged factor of substep i (made outside any capture: it
        allocates and copies its descriptors)."""
        sp = spec or P.RefineSpec()
        key = (i, sp.aiter, sp.siter, sp.diter, sp.tolsc)
        if key not in self.ragged_factors:
            self.ragged_factors[key] = P.RaggedFactor(
                self.plans, [self._phis(ci, i)[1] for ci in range(len(self.plans))], spec)
        return self.ragged_factors[key]

    def _issue_ragged(self, spec, substeps):
        """Per substep: every case's stage 1 on its stream, one ragged factor
        over all cases on the current stream, every case's stage 2."""
        torch = self.torch
        cur = torch.cuda.current_stream()
        for j, i in enumerate(substeps):
            rf = self._ragged_factor(i, spec)
            for stage in (1, 2):
                for s in self.streams:
                    s.wait_stream(cur)
                for ci, pl in enumerate(self.plans):
                    st = self.streams[ci % self.nstreams]
                    pe, pi = self._phis(ci, i)
                    a, b = self.bufs[ci][j % 2], self.bufs[ci][(j + 1) % 2]
                    with torch.cuda.stream(st):
                        pl.substep_stage(stage, pe, pi, a, b, spec, stream=st.cuda_stream)
                for s in self.streams:
                    cur.wait_stream(s)
                if stage == 1:
                    rf.factor(stream=cur.cuda_stream)

    def _issue(self, method, spec, substeps, capturable):
        """Every case's substeps on its stream (fork from / join into the
        current stream)."""
        torch = self.torch
        if self.ragged and capturable:
            if method != "M":
                raise ValueError("ragged mode runs the mixed method 'M' only")
            return self._issue_ragged(spec, substeps)
        cur = torch.cuda.current_stream()
        for s in self.streams:
            s.wait_stream(cur)
        for ci, pl in enumerate(self.plans):
            st = self.streams[ci % self.nstreams]
            with torch.cuda.stream(st):
                for j, i in enumerate(substeps):
                    pe, pi = self._phis(ci, i)
                    a, b = self.bufs[ci][j % 2], self.bufs[ci][(j + 1) % 2]
                    fn = pl.substep_capturable if capturable else pl.substep
                    fn(method, pe, pi, a, b, spec, stream=st.cuda_stream)
        for s in self.streams:
            cur.wait_stream(s)

    def reset(self) -> None:
        """State buffers back to the initial condition."""
        for du, b in zip(self.u0, self.bufs):
            b[0].copy_(du)

    def result(self, ci: int):
        """State of case ci after the last step (device tensor)."""
        return self.bufs[ci][self.nsubsteps % 2]

    def step_eager(self, method: str = "M", spec=None, substeps=(0, 1, 2)) -> None:
        """One step, host-driven (the reference path of the captured step)."""
        self.nsubsteps = len(substeps)
        self._issue(method, spec, substeps, capturable=False)

    def step_capturable(self, method: str = "M", spec=None, substeps=(0, 1, 2)) -> None:
        """One step in the captured step's form, issued directly (each plan
        must have run one ordinary substep of `method` first)."""
        self.nsubsteps = len(substeps)
        self._issue(method, spec, substeps, capturable=True)

    def capture(self, method: str = "M", spec=None, substeps=(0, 1, 2)) -> None:
        """Record one step (every case, the given substeps) into a CUDA graph.
        Each plan first runs one ordinary substep (allocation, one-time
        kernel attributes), outside the graph."""
        torch = self.torch
        self.reset()
        for ci, (c, pl) in enumerate(zip(self.configs, self.plans)):
            pe, pi = synth.smr91_phis(c.phi)
            pl.substep(method, pe, pi, self.bufs[ci][0], self.bufs[ci][1], spec)
        torch.cuda.synchronize()
        if self.ragged and method == "M":
            for i in substeps:
                self._ragged_factor(i, spec)
        self.reset()
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        L = self.plans[0].L
        l0 = L.sgb_launch_count()
        with torch.cuda.graph(self.graph):
            self._issue(method, spec, substeps, capturable=True)
        self.graph_kernels = int(L.sgb_launch_count() - l0)   # kernel nodes of one step
        self.nsubsteps = len(substeps)

    def replay(self) -> None:
        self.graph.replay()

    def unserved(self) -> int:
        return sum(p.unserved() for p in self.plans)

    def close(self) -> None:
        for rf in self.ragged_factors.values():
            rf.close()
        self.ragged_factors = {}

    def backward_error(self) -> np.ndarray:
        """Normwise backward error of the last substep of every system."""
        return np.concatenate([p.backward_error() for p in self.plans])
