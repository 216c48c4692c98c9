"""Host logic of the continuous-batching request loop (serve.Server.run),
without a GPU: streams, events, device buffers and plans are fakes that
model what the loop relies on (work on one stream runs in issue order; an
event completes when the work recorded before it on its stream has run; a
plan's substep advances the case's state), so that admission in arrival
order, the HBM budget, overlap of resident cases, the alternating state
buffers, plan release and latency accounting are checked on CPU, as are
the batch's row partition and MultiCase's SMR91
substep coefficients, stream assignment and state ping-pong.  The GPU counterpart
(test_serving_result_same_alone_and_in_the_mix) checks that each case's
result is the same alone and in the mix."""
import dataclasses
import sys
import time
import types

import numpy as np
import pytest

from suzerain_gb300 import serve


class _Arr(np.ndarray):
    def cuda(self):
        return self.copy()

    def cpu(self):
        return self

    def numpy(self):
        return np.asarray(self)


class _Device:
    def __init__(self):
        self.streams = {}
        self.log = []            # (rid, substep, start, end) per issued substep


class _Stream:
    def __init__(self, dev):
        self.cuda_stream = len(dev.streams) + 1
        self.busy_until = 0.0
        dev.streams[self.cuda_stream] = self


class _Event:
    def __init__(self, enable_timing=False):
        self.t = None

    def record(self, stream=None):
        now = time.perf_counter()
        self.t = max(now, stream.busy_until) if stream is not None else now

    def query(self):
        return time.perf_counter() >= self.t

    def elapsed_time(self, other):
        return (other.t - self.t) * 1e3


def _fake_torch(dev):
    class _StreamCtx:
        def __init__(self, st):
            self.st = st

        def __enter__(self):
            return self.st

        def __exit__(self, *a):
            return False

    cuda = types.SimpleNamespace(Stream=lambda: _Stream(dev), Event=_Event,
                                 synchronize=lambda: None, stream=_StreamCtx)
    return types.SimpleNamespace(cuda=cuda,
                                 from_numpy=lambda a: np.asarray(a).view(_Arr),
                                 empty_like=lambda a: np.empty_like(a).view(_Arr))


@dataclasses.dataclass
class _Case:
    rid: int
    nsys: int
    bytes: int
    dur: float
    phi: float = 1e-3

    def batch(self):
        cs = {"rid": self.rid, "bytes": self.bytes, "dur": self.dur}
        u = np.full((self.nsys, 4), float(self.rid), dtype=np.complex128)
        return cs, np.zeros(self.nsys), np.zeros(self.nsys), u


def _fake_plan(dev, created, closed):
    class Plan:
        def __init__(self, cs, kx, kz, max_double_slots=0):
            self.cs, self.nsys, self.k = cs, len(kx), 0
            created.append(cs["rid"])

        @staticmethod
        def estimate_bytes(cs, nsys, slots, method):
            return cs["bytes"]

        def prepare(self, method):
            pass

        def substep_capturable(self, method, pe, pi, a, b, spec, stream=0):
            st = dev.streams[stream]
            start = max(time.perf_counter(), st.busy_until)
            st.busy_until = start + self.cs["dur"]
            b[...] = a + 1
            dev.log.append((self.cs["rid"], self.k, start, st.busy_until))
            self.k += 1

        def close(self):
            closed.append(self.cs["rid"])

    return Plan


@pytest.fixture
def fake(monkeypatch):
    dev = _Device()
    created, closed = [], []
    monkeypatch.setitem(sys.modules, "torch", _fake_torch(dev))
    monkeypatch.setattr(serve.P, "Plan", _fake_plan(dev, created, closed))
    monkeypatch.setattr(serve.synth, "zero_dirichlet_rows", lambda cs, u: u)
    return types.SimpleNamespace(dev=dev, created=created, closed=closed)


def _trace(arrivals, lives, nbytes, dur, nsys=8):
    return [serve.Request(i, _Case(i, nsys, nbytes, dur), n, t)
            for i, (t, n) in enumerate(zip(arrivals, lives))]


def _need(srv, req):
    return srv._prepare(req)[-1]


def test_admission_in_arrival_order_within_budget_with_overlap(fake):
    arrivals = [0.0, 0.004, 0.008, 0.012, 0.03, 0.031, 0.05, 0.06]
    lives = [3, 4, 5, 3, 4, 3, 5, 3]
    trace = _trace(arrivals, lives, 30_000_000, 0.01)
    trace = trace[3:] + trace[:3]                  # the loop sorts by arrival
    srv = serve.Server(budget_bytes=100e6, nstreams=4, keep_results=True)
    need = _need(srv, trace[0])
    st = srv.run(trace)

    assert st["substeps"] == st["issued"] == sum(lives)
    assert st["system_solves"] == 8 * sum(lives)
    assert fake.created == sorted(fake.created) == list(range(8))
    assert sorted(fake.closed) == list(range(8))
    assert st["peak_resident_bytes"] <= 100e6
    assert st["peak_resident_bytes"] // need == 3   # three 30 MB cases fit
    assert st["peak_resident_cases"] >= 2
    for rid, n in enumerate(lives):                   # state advanced once per substep,
        np.testing.assert_array_equal(srv.results[rid], rid + n)   # buffers alternate
    # substeps of one case run one after another; different cases overlap
    spans = {}
    for rid, k, t0, t1 in fake.dev.log:
        spans.setdefault(rid, []).append((k, t0, t1))
    for rid, s in spans.items():
        assert [k for k, _, _ in s] == list(range(lives[rid]))
        assert all(b[1] >= a[2] - 1e-9 for a, b in zip(s, s[1:]))
    first = {rid: s[0][1] for rid, s in spans.items()}
    last = {rid: s[-1][2] for rid, s in spans.items()}
    assert any(first[j] < last[i] for i in spans for j in spans if j > i)
    assert st["p50_ms"] >= 0.9 * 10.0


def test_budget_of_one_case_serialises_cases_and_counts_their_wait(fake):
    trace = _trace([0.0, 0.0, 0.0], [3, 3, 3], 60_000_000, 0.01)
    srv = serve.Server(budget_bytes=100e6, nstreams=3)
    st = srv.run(trace)
    assert st["substeps"] == 9 and st["peak_resident_cases"] == 1
    spans = {}
    for rid, k, t0, t1 in fake.dev.log:
        spans.setdefault(rid, []).append((t0, t1))
    assert spans[1][0][0] >= spans[0][-1][1] - 1e-9
    assert spans[2][0][0] >= spans[1][-1][1] - 1e-9
    # the third case's first substep waited for six others: its latency
    # counts from arrival, so the p99 is well above one substep
    assert st["p99_ms"] >= 50.0
    assert st["queue_p99_ms"] >= 40.0


def test_case_larger_than_the_budget_runs_alone(fake):
    trace = _trace([0.0, 0.001], [2, 2], 150_000_000, 0.005)
    srv = serve.Server(budget_bytes=100e6, nstreams=2)
    st = srv.run(trace)
    assert st["substeps"] == 4 and st["peak_resident_cases"] == 1
    assert fake.closed == [0, 1]


def test_batch_bounds_partition_rows():
    """A batch's parts are consecutive row ranges, part i holding rows
    i n / parts .. (i + 1) n / parts - 1 (sgb_batch_bounds, host code), with
    the part count clamped to the systems; bad arguments are refused."""
    from suzerain_gb300 import plan as P
    assert P.bounds(10, 4) == [0, 2, 5, 7, 10]
    assert P.bounds(5, 8) == [0, 1, 2, 3, 4, 5]
    assert P.bounds(24768, 4) == [0, 6192, 12384, 18576, 24768]
    b = P.bounds(172160, 7)
    assert b[0] == 0 and b[-1] == 172160 and len(b) == 8
    sizes = np.diff(b)
    assert sizes.max() - sizes.min() <= 1
    with pytest.raises(ValueError):
        P.bounds(0, 4)
    with pytest.raises(ValueError):
        P.bounds(10, 0)

def test_multicase_step_scales_smr91_substeps_and_ping_pongs(monkeypatch):
    """MultiCase.step_eager issues every case's three SMR91 substeps in order
    on its stream (cases round-robin over the streams, forked from and joined
    into the caller's stream), with phi_explicit = dt alpha_i and
    phi_implicit = -dt beta_i for dt = phi / beta_0 (alpha = 29/96, -3/40,
    1/6; beta = 37/160, 5/24, 1/6; suzerain/lowstorage.hpp:1286-1304), and
    ping-pongs the state: substep j reads buffer j % 2 and writes the other,
    so the result after three substeps is buffer 1.  Cases are grouped by
    (N, KL, KU) for the tuner."""
    from suzerain_gb300 import multicase as MC
    events = []

    class Stream:
        n = 0

        def __init__(self):
            Stream.n += 1
            self.cuda_stream = Stream.n

        def wait_stream(self, other):
            events.append(("wait", self.cuda_stream, other.cuda_stream))

    caller = Stream()

    class Ctx:
        def __init__(self, st):
            self.st = st

        def __enter__(self):
            return self.st

        def __exit__(self, *a):
            return False

    class T:
        def __init__(self, a):
            self.a = a

        def cuda(self):
            return T(self.a.copy())

        def clone(self):
            return T(self.a.copy())

    cuda = types.SimpleNamespace(Stream=Stream, current_stream=lambda: caller, stream=Ctx)
    monkeypatch.setitem(sys.modules, "torch", types.SimpleNamespace(
        cuda=cuda, from_numpy=lambda a: T(np.asarray(a)),
        empty_like=lambda t: T(np.zeros_like(t.a))))

    class Plan:
        def __init__(self, cs, kx, kz, max_double_slots=0):
            self.cs, self.nsys = cs, len(kx)

        def substep(self, method, pe, pi, a, b, spec, stream=0):
            b.a[...] = a.a + 1
            events.append(("substep", self.cs.rid, stream, pe, pi, id(a), id(b)))

    monkeypatch.setattr(MC.P, "Plan", Plan)
    monkeypatch.setattr(MC.synth, "zero_dirichlet_rows", lambda cs, u: u)

    @dataclasses.dataclass
    class Cfg:
        rid: int
        N: int
        phi: float

        def batch(self, complex_coupling=False):
            cs = types.SimpleNamespace(rid=self.rid, N=self.N, KL=34, KU=34)
            return cs, np.zeros(4), np.zeros(4), np.full((4, self.N), float(self.rid))

    cfgs = [Cfg(0, 960, 1e-3), Cfg(1, 480, 2e-3), Cfg(2, 960, 1e-3)]
    mc = MC.MultiCase(cfgs, nstreams=2)
    assert mc.geometries() == {(960, 34, 34): [0, 2], (480, 34, 34): [1]}
    events.clear()
    mc.step_eager("M")
    part = [s.cuda_stream for s in mc.streams]
    assert events[:2] == [("wait", s, caller.cuda_stream) for s in part]
    assert events[-2:] == [("wait", caller.cuda_stream, s) for s in part]
    subs = [e for e in events if e[0] == "substep"]
    alpha, beta = (29 / 96, -3 / 40, 1 / 6), (37 / 160, 5 / 24, 1 / 6)
    for ci, cfg in enumerate(cfgs):
        mine = [e for e in subs if e[1] == ci]
        assert len(mine) == 3 and all(e[2] == part[ci % 2] for e in mine)
        dt = cfg.phi / beta[0]
        for i, e in enumerate(mine):
            assert np.isclose(e[3], dt * alpha[i], rtol=1e-15)
            assert np.isclose(e[4], -dt * beta[i], rtol=1e-15)
        b0, b1 = (id(x) for x in mc.bufs[ci])
        assert [(e[5], e[6]) for e in mine] == [(b0, b1), (b1, b0), (b0, b1)]
        np.testing.assert_array_equal(mc.result(ci).a, ci + 3)


def test_poisson_trace_matches_configuration_4():
    """Configuration 4's request stream: exponential inter-arrival times of
    mean 1/rate (arrivals increasing), case shapes drawn from configuration
    3's distribution (its own seeded set of cases unless a pool is given), lifetimes uniform on 3..30 substeps, each request its own
    seeded state, the same trace for the same seed."""
    from suzerain_gb300 import synth
    pool = synth.config3_cases()
    tr = serve.poisson_trace(4000, rate=100.0, seed=11)
    t = np.array([r.t_arrival for r in tr])
    assert (np.diff(t) > 0).all() and t[0] > 0
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(gaps.mean() - 0.01) < 0.001 and abs(gaps.std() - 0.01) < 0.0015
    lives = np.array([r.nsubsteps for r in tr])
    assert lives.min() == 3 and lives.max() == 30
    assert abs(lives.mean() - 16.5) < 0.6
    for r in tr:
        c = r.config
        assert c.Ny in range(32, 257, 16) and c.k in (6, 8) and c.S in (5, 7)
        assert (c.Nx, c.Nz) in ((32, 32), (64, 48), (128, 96))
    assert len({r.config.seed for r in tr}) == len(tr)
    assert [r.rid for r in tr] == list(range(len(tr)))
    again = serve.poisson_trace(4000, rate=100.0, seed=11)
    assert [(r.t_arrival, r.nsubsteps, r.config.Ny) for r in again] == \
        [(r.t_arrival, r.nsubsteps, r.config.Ny) for r in tr]
    short = serve.poisson_trace(50, rate=10.0, seed=3, configs=pool[:2], life=(4, 4))
    assert {r.nsubsteps for r in short} == {4}
    assert {r.config.Ny for r in short} <= {pool[0].Ny, pool[1].Ny}
