"""Many independent periodic IB problems stepped together.

``BatchedProblems`` packs any number of periodic problems of uneven grid
and marker sizes (same dimension and kernel) into one plan: one binning
sequence, one dense-tile spread, one per-visit spread and one interpolation
launch serve every problem, and the whole step (bin + spread + interpolate)
is captured once into a CUDA graph and replayed.  Grids live in one FP32
buffer per field, markers in one FP64 position buffer and FP32 value
buffers, every array starting on a 16-byte boundary.

This is the batched form of LEInteractor::spread / interpolate for
independent patches (ibtk/src/lagrangian/LEInteractor.cpp:3627-3714 and
2402-2489 applied patch by patch); each problem's results equal the
single-problem plan's within FP32 rounding.
"""

import numpy as np

from . import ibx


def _align(n, a=4):
    return (n + a - 1) // a * a


class BatchedProblems:
    """Periodic side-centred problems ``[(N, X), ...]`` with N a list of cells
    per axis and X the FP64 marker positions (numpy, d per marker)."""

    def __init__(self, problems, dim=2, kernel="IB_4", device="cuda", tune=True, tune_reps=3):
        import torch

        self.dim = dim
        self.kernel = kernel
        self.device = torch.device(device)
        self.sizes = [list(N) for N, _ in problems]
        self.n_markers = [X.size // dim for _, X in problems]
        # Packed layout: grid offsets (floats) per problem and component.
        goff, total = [], 0
        for N in self.sizes:
            vol = int(np.prod(N))
            offs = []
            for _ in range(dim):
                offs.append(total)
                total += _align(vol)
            goff.append(offs)
        self.grid_offsets = goff
        self.grid_values = total
        moff = np.concatenate([[0], np.cumsum(self.n_markers)]).astype(np.int64)
        self.marker_offsets = moff
        nm = int(moff[-1])
        f32 = dict(dtype=torch.float32, device=self.device)
        self.f = torch.zeros(total, **f32)       # spread target (force density)
        self.u = torch.zeros(total, **f32)       # interpolation source (velocity)
        self.X = torch.zeros(nm * dim, dtype=torch.float64, device=self.device)
        self.F = torch.zeros(nm * dim, **f32)    # marker forces
        self.U = torch.zeros(nm * dim, **f32)    # interpolated marker velocities
        self.X.copy_(torch.from_numpy(np.concatenate([X for _, X in problems])))
        sp, ip = [], []
        for k, N in enumerate(self.sizes):
            vol = int(np.prod(N))
            fq = [self.f[o:o + vol].view(N[::-1]) for o in goff[k]]
            uq = [self.u[o:o + vol].view(N[::-1]) for o in goff[k]]
            a, b = int(moff[k]) * dim, int(moff[k + 1]) * dim
            dx = [1.0 / n for n in N]
            mk = lambda q, Q: ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0] * dim, [n - 1 for n in N], dx,
                                               [0.0] * dim, [1.0] * dim, q, self.X[a:b], Q[a:b])
            sp.append(mk(fq, self.F))
            ip.append(mk(uq, self.U))
        self._make = lambda shape: ibx.Plan(sp, kernel, ibx.MIXED, interp_problems=ip, tile_shape=shape)
        self.tuning = None
        self.plan = None
        self.graph = None
        if tune:
            self.autotune(tune_reps)
        else:
            self.plan = self._make(0)

    def configure(self, setting):
        """Use a fixed setting (``tuning.parse_setting``): a plan of its tile
        shape with its knobs; a captured graph is dropped."""
        from . import tuning

        self._drop_graph()
        if self.plan is not None:
            self.plan.close()
        self.plan = self._make(setting.get("tile_shape", 0))
        tuning.apply_setting(self.plan, setting)

    def autotune(self, reps=3):
        """Tune the plan (tile shape and knobs, ``tuning.autotune_shape``) on
        the current contents of the buffers, which should hold representative
        forces and velocities: the kernels skip zero contributions.  The
        spread target ``f`` is zeroed afterwards; a captured graph is dropped."""
        from . import tuning

        self._drop_graph()
        if self.plan is not None:
            self.plan.close()
        self.plan, self.tuning = tuning.autotune_shape(self._make, reps=reps)
        self.f.zero_()

    # -- views ------------------------------------------------------------
    def grid(self, field, k):
        """The d arrays (one per side axis) of problem k of ``self.f`` / ``self.u``."""
        vol = int(np.prod(self.sizes[k]))
        buf = self.f if field == "f" else self.u
        return [buf[o:o + vol].view(self.sizes[k][::-1]) for o in self.grid_offsets[k]]

    def markers(self, buf, k):
        a, b = int(self.marker_offsets[k]) * self.dim, int(self.marker_offsets[k + 1]) * self.dim
        return buf[a:b]

    # -- stepping ----------------------------------------------------------
    def step(self, io=None):
        """bin, then spread (f += S F) and interpolate (U = S* u)
        concurrently, eagerly.  io: host transfers around the step, a dict of
        Plan.step_io's in_X / in_Q / out_Q lists of (dst, src) pairs."""
        if io:
            self.plan.step_io(**io)
        else:
            self.plan.step()

    def host_io(self, Xh, Fh, Uh):
        """The transfers of a step whose positions Xh and forces Fh come from
        pinned host tensors and whose velocities go to the pinned host tensor
        Uh (all batch-wide, the layout of X, F and U)."""
        return dict(in_X=[(self.X, Xh)], in_Q=[(self.F, Fh)], out_Q=[(Uh, self.U)])

    def capture(self, io=None):
        """Capture one step (with the host transfers io, see step) into a
        CUDA graph that keeps the plan's stream priorities (Plan.graph),
        after an eager warm-up step."""
        import torch

        self._drop_graph()
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.step(io)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        self.graph = self.plan.graph(**(io or {}))
        return self.graph

    def replay(self, stream=None):
        if self.graph is None:
            self.capture()
        self.graph.launch(stream)

    def _drop_graph(self):
        if self.graph is not None:
            self.graph.close()
        self.graph = None

    def status(self):
        return self.plan.status()

    def close(self):
        self._drop_graph()
        self.plan.close()
