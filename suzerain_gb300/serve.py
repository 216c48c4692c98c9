"""Continuous-batching request loop for substep solves (configuration 4).

A request is one case (its S, Ny, k and wavenumber grid) that lives for a
given number of SMR91 substeps.  Requests arrive over time; the loop

* admits waiting requests in arrival order while the device bytes of the
  resident cases plus the new case's estimate (``Plan.estimate_bytes``) stay
  within the HBM budget, creating the case's plan and uploading its state;
* issues each resident case's next substep as soon as its previous one
  completes (a CUDA event per case, polled), on streams shared round-robin,
  so that the cases' work overlaps on the device and requests admitted while
  others run start at once (continuous batching, not a queue);
* keeps each case's factors, refinement state and solution resident between
  its substeps, and frees the plan when its last substep completes.

Latency of a substep = completion time - the time it became ready (arrival
for a case's first substep, the completion of its previous substep
otherwise); completion times come from CUDA events recorded after each
case's substep.  A case's results do not depend on which other cases share
its ticks: each plan owns all of its buffers and the kernels are
deterministic.
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np

from . import plan as P
from . import synth


@dataclasses.dataclass
class Request:
    rid: int
    config: object            # synth.Config
    nsubsteps: int
    t_arrival: float          # seconds from the start of the run


@dataclasses.dataclass
class _Live:
    req: Request
    plan: object
    bufs: list
    bytes: int
    done: int = 0
    t_ready: float = 0.0
    stream: object = None
    event: object = None


def poisson_trace(nreq: int, rate: float, seed: int, configs=None,
                  life=(3, 30)) -> list[Request]:
    """nreq requests with exponential inter-arrival times of mean 1/rate,
    case shapes drawn from configuration 3's distribution, lifetimes uniform
    on life (inclusive)."""
    rng = np.random.default_rng(seed)
    pool = configs or synth.config3_cases(64, seed=synth.SEED_BASE + 4)
    t, out = 0.0, []
    for i in range(nreq):
        t += float(rng.exponential(1.0 / rate))
        c = pool[int(rng.integers(len(pool)))]
        c = dataclasses.replace(c, name=f"req{i}", seed=synth.SEED_BASE * 7 + i)
        out.append(Request(i, c, int(rng.integers(life[0], life[1] + 1)), t))
    return out


class Server:
    def __init__(self, budget_bytes: float = 120e9, method: str = "M", spec=None,
                 nstreams: int = 16, max_double_slots: int = 128, keep_results: bool = False):
        import torch
        self.torch = torch
        self.budget = float(budget_bytes)
        self.method = method
        self.spec = spec or P.RefineSpec(aiter=5, siter=25, diter=5, tolsc=145.0)
        self.streams = [torch.cuda.Stream() for _ in range(max(1, nstreams))]
        self.max_double_slots = max_double_slots
        self.keep_results = keep_results
        self.results = {}

    def _prepare(self, req: Request):
        """Host-side case construction (bands, wavenumbers, initial state)
        and the device bytes the case will hold; cached on the request."""
        if getattr(req, "_built", None) is None:
            cs, kx, kz, u = req.config.batch()
            synth.zero_dirichlet_rows(cs, u)
            slots = min(self.max_double_slots, len(kx))
            need = P.Plan.estimate_bytes(cs, len(kx), slots, self.method) + 2 * u.size * 16
            req._built = (cs, kx, kz, u, slots, need)
        return req._built

    def prebuild(self, trace: list[Request]) -> None:
        """Build every request's host-side case and state before the run (a
        client hands the server its state; generating it is not serving)."""
        for r in trace:
            self._prepare(r)

    def _admit(self, req: Request, now: float) -> _Live:
        torch = self.torch
        cs, kx, kz, u, slots, need = self._prepare(req)
        pl = P.Plan(cs, kx, kz, max_double_slots=slots)
        pl.prepare(self.method)
        du = torch.from_numpy(u).cuda()
        req._built = None
        return _Live(req, pl, [du, torch.empty_like(du)], need, 0, now)

    def run(self, trace: list[Request]) -> dict:
        """Serve the trace in real time; returns latency and throughput
        statistics (latencies in ms).  Each resident case advances on its own:
        its next substep is issued as soon as its previous one completes, and
        arrivals are admitted between any two completions."""
        torch = self.torch
        pending = sorted(trace, key=lambda r: r.t_arrival)
        live: list[_Live] = []
        used = 0
        lat, qwait, solves, issued = [], [], 0, 0
        peak_live, peak_bytes = 0, 0
        ref = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ref.record()
        clock = lambda: time.perf_counter() - t0
        nst = len(self.streams)

        def issue(lv: _Live):
            nonlocal issued
            c = lv.req.config
            i = lv.done % 3
            pe, pi_ = synth.smr91_phis(c.phi * synth.SMR91_BETA[i] / synth.SMR91_BETA[0],
                                       substep=i)
            a, b = lv.bufs[lv.done % 2], lv.bufs[(lv.done + 1) % 2]
            st = lv.stream
            with torch.cuda.stream(st):
                # no host synchronization inside: the cases' substeps overlap
                lv.plan.substep_capturable(self.method, pe, pi_, a, b, self.spec,
                                           stream=st.cuda_stream)
                lv.event = torch.cuda.Event(enable_timing=True)
                lv.event.record(st)
            issued += 1

        pi = 0
        while pi < len(pending) or live:
            now = clock()
            # admission in arrival order, against the memory budget
            while pi < len(pending) and pending[pi].t_arrival <= now:
                req = pending[pi]
                need = self._prepare(req)[-1]
                if live and used + need > self.budget:
                    break           # wait for resident cases to finish
                lv = self._admit(req, now)
                lv.t_ready = req.t_arrival
                lv.stream = self.streams[req.rid % nst]
                qwait.append((clock() - req.t_arrival) * 1e3)
                live.append(lv)
                used += lv.bytes
                pi += 1
                issue(lv)
            peak_live = max(peak_live, len(live))
            peak_bytes = max(peak_bytes, used)
            progressed = False
            still = []
            for lv in live:
                if not lv.event.query():
                    still.append(lv)
                    continue
                progressed = True
                t_done = ref.elapsed_time(lv.event) / 1e3
                lat.append((t_done - lv.t_ready) * 1e3)
                solves += lv.plan.nsys
                lv.done += 1
                lv.t_ready = t_done
                if lv.done >= lv.req.nsubsteps:
                    if self.keep_results:
                        self.results[lv.req.rid] = lv.bufs[lv.done % 2].cpu().numpy()
                    used -= lv.bytes
                    lv.plan.close()
                else:
                    issue(lv)
                    still.append(lv)
            live = still
            if not progressed:
                nxt = pending[pi].t_arrival - clock() if pi < len(pending) else 1.0
                time.sleep(max(0.0, min(nxt, 2e-4)))
        wall = clock()
        lat = np.asarray(lat)
        return {"requests": len(trace), "substeps": int(lat.size), "issued": issued,
                "wall_s": wall, "system_solves": solves, "throughput": solves / wall,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "queue_p99_ms": float(np.percentile(qwait, 99)) if qwait else 0.0,
                "peak_resident_cases": peak_live, "peak_resident_bytes": int(peak_bytes)}
