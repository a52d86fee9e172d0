"""Request loop over resident IB simulations on one GPU.

A request asks for one spread + interpolate step of a resident simulation
(its markers, force and velocity fields and binning plan stay on the
device).  The loop is continuous batching over CUDA streams: requests that
arrive while others are running are admitted as soon as a slot (stream) is
free and the simulation they address is not already running, so work from
different requests overlaps on the device; a request whose simulation is
not resident is admitted once the HBM budget allows creating it, evicting
idle simulations in least-recently-used order.  Each request's latency is
measured from its arrival to the host observing its completion event.

The scheduler is written against a small backend interface so that its
logic runs on the CPU in tests (``FakeBackend``) and on the GPU through
``CudaBackend``.
"""

import collections
import time

import numpy as np

from . import ibx


# ---------------------------------------------------------------------------
# Memory estimate of one simulation (device bytes), used for admission.
# ---------------------------------------------------------------------------
def plan_bytes_estimate(dim, N, n_markers):
    """Upper bound of ibx_plan_scratch_bytes for one periodic problem: the
    buffers of the plan (records in two orders, lists, home units, counters,
    work items), with the visit capacity the library reserves."""
    E = 8 if dim == 3 else 16
    tiles = int(np.prod([(n + E - 1) // E for n in N]))
    per = 1
    for n in N:
        nt = (n + E - 1) // E
        per *= min(nt, 2 + (n % E != 0))
    visit_cap = n_markers * per
    b = 0
    b += 2 * 32 * n_markers                     # records (marker order, home order)
    b += 3 * 4 * n_markers + 8 * n_markers      # home tile, home list, home units
    b += visit_cap * 4                          # visit list
    b += 4 * (7 * tiles + 4)                    # counters
    b += 4 * (tiles + n_markers // 10 + 1)      # dense work items
    b += 4 * 2 * 2048 + 4096 + 13 * 256         # scan scratch, descriptors, alignment
    return b


def simulation_bytes(dim, N, n_markers):
    """Device bytes of a resident simulation: FP32 force and velocity side
    fields, FP64 positions, FP32 forces and velocities, plan scratch."""
    vol = int(np.prod(N))
    return 2 * dim * vol * 4 + n_markers * dim * (8 + 4 + 4) + plan_bytes_estimate(dim, N, n_markers)


class SimSpec:
    """A simulation known to the server: geometry, markers, forces and
    velocity field (host arrays, uploaded when it becomes resident)."""

    def __init__(self, sid, dim, N, X, F=None, u=None):
        self.sid = sid
        self.dim = dim
        self.N = list(N)
        self.X = X
        self.F = F
        self.u = u
        self.n_markers = X.size // dim
        self.bytes = simulation_bytes(dim, N, self.n_markers)


# ---------------------------------------------------------------------------
# Backends
# ---------------------------------------------------------------------------
class CudaBackend:
    """Resident simulations on the current CUDA device; one stream per slot.
    With ``graphs`` each simulation's step is captured into a CUDA graph when
    it becomes resident and a request replays it (one launch instead of the
    step's kernels, no per-request host work beyond that)."""

    def __init__(self, kernel="IB_4", device="cuda", graphs=True):
        import torch

        self.torch = torch
        self.kernel = kernel
        self.device = torch.device(device)
        self.graphs = graphs
        self.kernel_launches = 0  # library kernels run by launch(), graph nodes included

    def make_slots(self, n):
        return [self.torch.cuda.Stream(device=self.device) for _ in range(n)]

    def create(self, spec):
        sim = _CudaSim(spec, self.kernel, self.device)
        if self.graphs:
            sim.capture()
        return sim

    def launch(self, sim, slot, keep=False):
        """One step of ``sim`` on stream ``slot``; returns (event, results)
        where results are copies of (U, f) taken on the same stream when
        ``keep`` is set."""
        torch = self.torch
        with torch.cuda.stream(slot):
            if sim.graph is not None:
                sim.graph.replay()
                self.kernel_launches += sim.kernels_per_step
            else:
                l0 = ibx.kernel_launches()
                sim.step(slot)
                self.kernel_launches += ibx.kernel_launches() - l0
            res = None
            if keep:
                res = (sim.U.clone(), [t.clone() for t in sim.f])
            ev = torch.cuda.Event()
            ev.record(slot)
        return ev, res

    def done(self, handle):
        return handle.query()

    def destroy(self, sim):
        sim.close()


class _CudaSim:
    def __init__(self, spec, kernel, device):
        import torch

        dim, N = spec.dim, spec.N
        f32 = dict(dtype=torch.float32, device=device)
        shape = N[::-1]
        self.f = [torch.zeros(shape, **f32) for _ in range(dim)]
        if spec.u is not None:
            self.u = [torch.tensor(spec.u[a], **f32) for a in range(dim)]
        else:
            self.u = [torch.zeros(shape, **f32) for _ in range(dim)]
        self.X = torch.tensor(spec.X, dtype=torch.float64, device=device)
        F = spec.F if spec.F is not None else np.zeros(spec.X.size)
        self.F = torch.tensor(F, **f32)
        self.U = torch.zeros(spec.X.size, **f32)
        dx = [1.0 / n for n in N]
        mk = lambda q, Q: ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0] * dim, [n - 1 for n in N], dx,
                                           [0.0] * dim, [1.0] * dim, q, self.X, Q)
        self.plan = ibx.Plan(mk(self.f, self.F), kernel, ibx.MIXED, interp_problems=[mk(self.u, self.U)])
        self.n_markers = spec.n_markers
        self.graph = None
        self.kernels_per_step = 0  # library kernels in one step (counted at capture)
        # the uploads and fills above ran on the current stream; the steps
        # run on slot streams
        torch.cuda.current_stream().synchronize()

    def step(self, stream):
        for t in self.f:
            t.zero_()
        self.plan.step(stream)

    def capture(self):
        """Capture one step into a CUDA graph (after an eager warm-up)."""
        import torch

        s = torch.cuda.Stream(device=self.X.device)
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.step(s)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        l0 = ibx.kernel_launches()
        with torch.cuda.graph(g):
            self.step(torch.cuda.current_stream())
        self.kernels_per_step = ibx.kernel_launches() - l0
        torch.cuda.synchronize()
        self.graph = g

    def close(self):
        self.graph = None
        self.plan.close()


class FakeBackend:
    """Host-only stand-in for tests of the scheduler: a step of a simulation
    "runs" for duration(spec) seconds of wall time after its launch, and its
    result is a deterministic function of the simulation and the request."""

    def __init__(self, duration=lambda spec: 1e-4, clock=time.perf_counter):
        self.duration = duration
        self.clock = clock
        self.created = []
        self.destroyed = []
        self.launches = []

    def make_slots(self, n):
        return list(range(n))

    def create(self, spec):
        self.created.append(spec.sid)
        return spec

    def launch(self, sim, slot, keep=False):
        t = self.clock()
        self.launches.append((sim.sid, slot, t))
        res = ("result", sim.sid) if keep else None
        return t + self.duration(sim), res

    def done(self, handle):
        return self.clock() >= handle

    def destroy(self, sim):
        self.destroyed.append(sim.sid)


# ---------------------------------------------------------------------------
# The request loop
# ---------------------------------------------------------------------------
Request = collections.namedtuple("Request", "rid arrival sid")


def poisson_requests(rate, n, sids, seed=0):
    """n requests with exponential inter-arrival times (mean 1/rate seconds),
    each for a simulation drawn uniformly from sids."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    who = rng.choice(len(sids), size=n)
    return [Request(i, float(t[i]), sids[who[i]]) for i in range(n)]


class Server:
    """Continuous-batching request loop with HBM-budget admission."""

    def __init__(self, backend, budget_bytes, n_slots=8):
        self.backend = backend
        self.budget = int(budget_bytes)
        self.slots = backend.make_slots(n_slots)
        self.specs = {}
        self.resident = collections.OrderedDict()  # sid -> sim, least recently used first
        self.used = 0
        self.busy = set()
        self.evictions = 0

    def register(self, spec):
        if spec.bytes > self.budget:
            raise ValueError("simulation %r needs %d bytes, above the budget" % (spec.sid, spec.bytes))
        self.specs[spec.sid] = spec

    def _admit(self, sid):
        """Make sid resident if the budget allows (evicting idle simulations,
        least recently used first); False when it must wait."""
        if sid in self.resident:
            self.resident.move_to_end(sid)
            return True
        need = self.specs[sid].bytes
        if self.used + need > self.budget:
            idle = [s for s in self.resident if s not in self.busy]
            freeable = sum(self.specs[s].bytes for s in idle)
            if self.used - freeable + need > self.budget:
                return False
            for s in idle:
                if self.used + need <= self.budget:
                    break
                self.backend.destroy(self.resident.pop(s))
                self.used -= self.specs[s].bytes
                self.evictions += 1
        self.resident[sid] = self.backend.create(self.specs[sid])
        self.used += need
        return True

    def run(self, requests, keep_results=False, clock=time.perf_counter, time_scale=1.0):
        """Serve the requests (arrival times in seconds from the start);
        returns a dict of per-request latencies and totals."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        pending = collections.deque()
        free = list(range(len(self.slots)))
        in_flight = {}
        lat = {}
        results = {}
        done_markers = 0
        nxt = 0
        max_queue = 0
        t0 = clock()
        last_done = t0
        while len(lat) < len(reqs):
            now = clock() - t0
            while nxt < len(reqs) and reqs[nxt].arrival * time_scale <= now:
                pending.append(reqs[nxt])
                nxt += 1
            max_queue = max(max_queue, len(pending))
            for slot in list(in_flight):
                req, handle, res = in_flight[slot]
                if self.backend.done(handle):
                    t = clock()
                    lat[req.rid] = t - t0 - req.arrival * time_scale
                    last_done = t
                    done_markers += self.specs[req.sid].n_markers
                    if keep_results:
                        results[req.rid] = res
                    self.busy.discard(req.sid)
                    free.append(slot)
                    del in_flight[slot]
            # Dispatch in arrival order; a request whose simulation is running
            # or cannot be admitted yet lets later requests go ahead.
            if free and pending:
                waiting = collections.deque()
                while pending and free:
                    req = pending.popleft()
                    if req.sid in self.busy or not self._admit(req.sid):
                        waiting.append(req)
                        continue
                    slot = free.pop()
                    handle, res = self.backend.launch(self.resident[req.sid], self.slots[slot], keep=keep_results)
                    self.busy.add(req.sid)
                    in_flight[slot] = (req, handle, res)
                waiting.extend(pending)
                pending = waiting
        lats = np.array([lat[r.rid] for r in reqs])
        span = max(last_done - t0 - reqs[0].arrival * time_scale, 1e-12)
        out = {
            "requests": len(reqs),
            "latency_s": lat,
            "p50_ms": float(np.percentile(lats, 50) * 1e3),
            "p99_ms": float(np.percentile(lats, 99) * 1e3),
            "mean_ms": float(lats.mean() * 1e3),
            "markers_per_s": done_markers / span,
            "requests_per_s": len(reqs) / span,
            "max_queue": max_queue,
            "evictions": self.evictions,
            "resident": len(self.resident),
            "used_bytes": self.used,
        }
        if keep_results:
            out["results"] = results
        return out

    def close(self):
        for sid in list(self.resident):
            self.backend.destroy(self.resident.pop(sid))
        self.used = 0
