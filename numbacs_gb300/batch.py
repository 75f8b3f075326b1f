"""Many FTLE fields in one CUDA graph.

The reference builds FTLE time series with a Python loop over t0 that calls
``flowmap_grid_2D`` and ``ftle_grid_2D`` per field
(examples/time_series/plot_dg_time_series.py,
examples/time_series/plot_dg_numbacs_vs_scipy.py).  :class:`FTLEBatch` takes
the whole list of fields -- any mix of flows, start times, integration
lengths and grid sizes -- and runs them under one of three schedules: one
persistent kernel whose warps take 32-particle chunks from a shared counter
(csrc/batch32.cu, csrc/batch64.cu); or per flow class (the fields that share
one right-hand side) one launch of a tile kernel with the single-field
integrator's block shape and register budget, one block per particle tile of
the class's fields, longest fields first, the classes on parallel streams;
each followed by one FTLE/eigenvector launch for all fields; or every field's
own single-field integrator and FTLE launches spread over parallel streams,
longest first, so that the tail of one field overlaps the start of the next.
The run is kernel launches only, so it is captured once in a CUDA graph and
replayed.
"""
import ctypes

import numpy as np
import torch

from . import _device as D
from . import _lib
from .flows import _check_callable_flow

_PREC = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}


class Field:
    """One FTLE field: the arguments of one flowmap_grid_2D call plus FTLE."""

    def __init__(self, flow, t0, T, x, y, params, rtol=1e-6, atol=1e-8, mask=None, ftle=True,
                 out=None):
        """``out``: an optional contiguous float64 (nx, ny, 2) CUDA tensor that
        receives the flow map (e.g. one slice of a stack of maps)."""
        self.flow = _check_callable_flow(flow)
        self.t0, self.T = float(t0), float(T)
        self.x, self.y = D.to_dev(x), D.to_dev(y)
        self.params = np.ascontiguousarray(
            params.cpu().numpy() if isinstance(params, torch.Tensor) else params, dtype=np.float64)
        if not 1 <= len(self.params) <= _lib.MAX_PARAMS:
            raise ValueError("params: 1..%d values" % _lib.MAX_PARAMS)
        self.rtol, self.atol = float(rtol), float(atol)
        self.mask = D.mask_to_dev(mask)
        self.want_ftle = bool(ftle)
        nx, ny = self.x.numel(), self.y.numel()
        if out is None:
            self.flowmap = D.empty((nx, ny, 2))
        elif (tuple(out.shape) != (nx, ny, 2) or out.dtype != torch.float64 or not out.is_cuda
              or not out.is_contiguous()):
            raise ValueError("out must be a contiguous float64 (nx, ny, 2) CUDA tensor")
        else:
            self.flowmap = out
        self.status = D.empty((nx, ny), torch.int32)
        self.ftle = D.empty((nx, ny)) if ftle else None
        self.evec = D.empty((nx, ny, 2)) if ftle else None
        # the grid spacing only enters the FTLE (read on the host: a sync)
        self.dx = self.dy = 1.0
        if ftle:
            xs = self.x.cpu()
            ys = self.y.cpu()
            self.dx = float(xs[1] - xs[0]) if nx > 1 else 1.0
            self.dy = float(ys[1] - ys[0]) if ny > 1 else 1.0

    @property
    def particles(self):
        return self.x.numel() * self.y.numel()


TILES = -1    # schedule: per flow class one tile kernel (classes on parallel streams)
STREAMS = -2  # schedule: one integrator + one FTLE launch per field on parallel streams


class FTLEBatch:
    """A prepared batch of fields; ``run()`` recomputes every field in place.

    ``precision`` is "mixed" or "fp64"; ``blocks_per_sm`` picks the schedule:
    >= 0 a persistent grid of that many blocks per SM (0: full occupancy) whose
    warps take particle chunks from a shared counter, -1 (``TILES``, mixed)
    per flow class one launch of the single-field integrator's block shape
    over the tiles of the class's fields, longest field first, the classes on
    parallel streams, -2 (``STREAMS``) each field's own single-field
    integrator and FTLE launches, spread longest first over ``max_streams``
    streams so that one field's tail overlaps the next field's start; None
    takes it from the autotuner cache, tuning on first use.  ``graph=True``
    captures the run (all streams) in a CUDA graph on first call.
    """

    def __init__(self, fields, precision="mixed", blocks_per_sm=None, graph=True, max_steps=100000,
                 max_streams=16):
        D.require_cuda()
        if precision not in _PREC:
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.fields = list(fields)
        if not self.fields:
            raise ValueError("empty batch")
        self.precision = precision
        flows, index = [], {}
        for f in self.fields:
            if id(f.flow) not in index:
                index[id(f.flow)] = len(flows)
                flows.append(f.flow)
        self._flows = flows
        FlowArr = _lib.NbcsFlow * len(flows)
        self._flow_arr = FlowArr(*[fl.struct for fl in flows])
        FieldArr = _lib.NbcsField * len(self.fields)
        arr = FieldArr()
        for k, f in enumerate(self.fields):
            s = arr[k]
            s.flow = index[id(f.flow)]
            s.nx, s.ny = f.x.numel(), f.y.numel()
            s.np = len(f.params)
            for q, v in enumerate(f.params):
                s.params[q] = float(v)
            s.t0, s.T, s.rtol, s.atol, s.dx, s.dy = f.t0, f.T, f.rtol, f.atol, f.dx, f.dy
            s.x, s.y = f.x.data_ptr(), f.y.data_ptr()
            s.mask = f.mask.data_ptr() if f.mask is not None else None
            s.flowmap, s.status = f.flowmap.data_ptr(), f.status.data_ptr()
            s.ftle = f.ftle.data_ptr() if f.ftle is not None else None
            s.evec_max = f.evec.data_ptr() if f.evec is not None else None
        self._field_arr = arr
        L = _lib.load()
        # the batched kernels take spline flows with extrap_mode "constant" only;
        # a batch holding another mode runs every field through its own launches
        self.kernels_ok = all(fl.kind != _lib.FLOW_SPLINE2D or fl.extrap == 0 for fl in flows)
        self.plan = _lib.NbcsBatch()
        self._scratch = None
        if self.kernels_ok:
            nbytes = L.nbcs_batch_scratch_bytes(len(flows), len(self.fields))
            self._scratch = torch.empty(nbytes, dtype=torch.uint8, device=D.device())
            _lib.check(L.nbcs_batch_prepare(self._flow_arr, len(flows), self._field_arr,
                                            len(self.fields), _PREC[precision],
                                            D.ptr(self._scratch), nbytes,
                                            ctypes.byref(self.plan), D.stream_ptr()))
        elif blocks_per_sm is not None and int(blocks_per_sm) != STREAMS:
            raise ValueError("a batch with extrap_mode 'nearest' or 'linear' flows runs only "
                             "the per-field schedule (blocks_per_sm=%d)" % STREAMS)
        else:
            blocks_per_sm = STREAMS
        self.max_steps = int(max_steps)
        self.max_streams = max(1, int(max_streams))
        self._streams = None
        self._class_streams = None
        self.tuning = None  # the autotuner's timings of the schedules, when it chose
        # longest work first: particles x |T|
        self._order = sorted(range(len(self.fields)),
                             key=lambda k: -self.fields[k].particles * abs(self.fields[k].T))
        if blocks_per_sm is None:
            from .autotune import tune_batch
            blocks_per_sm = tune_batch(self)
        self.blocks_per_sm = int(blocks_per_sm)
        self.use_graph = graph
        self._graph = None

    @property
    def particles(self):
        return sum(f.particles for f in self.fields)

    def _opts(self, blocks_per_sm=None):
        o = _lib.NbcsOpts()
        o.precision = _PREC[self.precision]
        o.max_steps = self.max_steps
        o.blocks_per_sm = self.blocks_per_sm if blocks_per_sm is None else int(blocks_per_sm)
        return o

    def launch(self, blocks_per_sm=None):
        """Enqueue one run on the current stream (no graph)."""
        bps = self.blocks_per_sm if blocks_per_sm is None else int(blocks_per_sm)
        if bps == STREAMS:
            self._launch_streams()
            return
        if bps == TILES and self.precision == "mixed" and self.plan.nclasses > 1:
            self._launch_classes()
            return
        _lib.check(_lib.load().nbcs_batch_run(ctypes.byref(self.plan), self._opts(blocks_per_sm),
                                              D.stream_ptr()))

    def _launch_classes(self):
        """The tile kernel of each flow class on its own stream (forked from and
        joined back into the current stream, capturable), then one FTLE launch
        for every field."""
        L = _lib.load()
        main = torch.cuda.current_stream()
        n = self.plan.nclasses
        if self._class_streams is None:
            self._class_streams = [torch.cuda.Stream() for _ in range(n)]
        o = self._opts(TILES)
        for k, s in enumerate(self._class_streams):
            s.wait_stream(main)
            _lib.check(L.nbcs_batch_run_class(ctypes.byref(self.plan), k, o,
                                              ctypes.c_void_p(s.cuda_stream)))
        for s in self._class_streams:
            main.wait_stream(s)
        _lib.check(L.nbcs_batch_run_ftle(ctypes.byref(self.plan), D.stream_ptr()))

    def _launch_streams(self):
        """Every field through the single-field entry points (nbcs_flowmap_grid_2d,
        nbcs_ftle_evec_2d) on its own stream of a small pool, forked from and
        joined back into the current stream (capturable)."""
        L = _lib.load()
        main = torch.cuda.current_stream()
        if self._streams is None:
            self._streams = [torch.cuda.Stream() for _ in
                             range(min(self.max_streams, len(self.fields)))]
        for s in self._streams:
            s.wait_stream(main)
        o = _lib.NbcsOpts()
        o.precision = _PREC[self.precision]
        o.max_steps = self.max_steps
        # two lanes a spline particle in the mixed path, as the other schedules
        # (the lane count sets the FP32 summation order): identical results
        o.lanes_per_particle = 2
        for q, k in enumerate(self._order):
            f = self.fields[k]
            sp = ctypes.c_void_p(self._streams[q % len(self._streams)].cuda_stream)
            nx, ny = f.x.numel(), f.y.numel()
            _lib.check(L.nbcs_flowmap_grid_2d(
                f.flow.struct, f.t0, f.T, D.ptr(f.x), nx, D.ptr(f.y), ny,
                f.params.ctypes.data_as(_lib._vp), len(f.params), f.rtol, f.atol, D.ptr(f.mask),
                D.ptr(f.flowmap), D.ptr(f.status), o, sp))
            if f.ftle is not None:
                _lib.check(L.nbcs_ftle_evec_2d(D.ptr(f.flowmap), nx, ny, f.T, f.dx, f.dy,
                                               D.ptr(f.mask), D.ptr(f.ftle), D.ptr(f.evec), sp))
        for s in self._streams:
            main.wait_stream(s)

    def capture(self):
        """Capture one run into a CUDA graph (after one eager warm-up run)."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.launch()
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch()
        self._graph = g
        return g

    def run(self):
        """Recompute every field (graph replay when enabled)."""
        if self.use_graph:
            if self._graph is None:
                self.capture()
            self._graph.replay()
        else:
            self.launch()
        return self

    def results(self):
        """[(flowmap, ftle, evec_max, status)] device tensors, one per field."""
        return [(f.flowmap, f.ftle, f.evec, f.status) for f in self.fields]
