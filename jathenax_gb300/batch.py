"""Batches: many independent device-resident solves advanced together.

Per RK stage, one persistent launch per (precision, reconstruction, Riemann
solver, kernel) group walks a tile work list spanning every grid of the
group, the groups of a stage running concurrently on side streams; the
batched begin-step kernel picks each solve's own dt; the forced solves of
one precision share one render launch and one normalise/kick sequence. A
whole cycle is enqueued by one ``jx_batch_step`` call and can be captured in
a CUDA graph. Each solve keeps its own clock, workspace and CFL partials
(one slot per tile), so a solve's result is bitwise the same alone and in
any batch.
"""

import ctypes

from . import _lib


class ClockBank:
    """One device buffer holding the 128-byte clocks of many solves."""

    def __init__(self, n):
        t = _lib.torch()
        self.buf = t.zeros((n, 128), dtype=t.uint8, device=_lib.device())
        self._host = None
        self._turn = 0

    def slot(self, i):
        return self.buf[i]

    def read(self):
        """Every clock, now (synchronises with the device)."""
        return self.parse(self.buf.cpu())

    def snapshot(self):
        """Enqueue a copy of every clock into pinned host memory.

        Returns (event, host): once the event has completed, ``parse(host)``
        gives the clocks as of this point of the stream. Two host buffers
        alternate, so a snapshot stays readable while the next one is copied.
        """
        t = _lib.torch()
        if self._host is None:
            self._host = [t.empty(self.buf.shape, dtype=t.uint8).pin_memory() for _ in range(2)]
        host = self._host[self._turn]
        self._turn ^= 1
        host.copy_(self.buf, non_blocking=True)
        event = t.cuda.Event(enable_timing=True)
        event.record()
        return event, host

    @staticmethod
    def parse(host):
        raw = host.numpy()
        return [_lib.Clock.from_buffer_copy(raw[i].tobytes()) for i in range(raw.shape[0])]


class Batch:
    """Advance a list of :class:`jathenax_gb300.solver.Solve` together.

    Solves have 3 or 4 variables; each keeps its own tile (the default, or
    ``tile=(32, h)`` / ``tile=(58, h)`` at construction).
    """

    def __init__(self, solves, blocks_per_sm=0, clocks=None):
        t = _lib.torch()
        self.solves = list(solves)
        if not self.solves:
            raise ValueError("a batch needs at least one solve")
        self.blocks_per_sm = int(blocks_per_sm)
        self.clocks = clocks
        n = len(self.solves)
        arr = (_lib.SolveStruct * n)(*[s.as_jx_solve() for s in self.solves])
        size = ctypes.c_size_t()
        _lib.call("jx_batch_plan_bytes", arr, n, ctypes.byref(size))
        nbytes = int(size.value)
        # Each plan gets its own buffers from torch's caching allocators: the
        # pinned host block is not handed out again until the asynchronous
        # copy below has run, and the device block is reused only in stream
        # order. (Rewriting one pinned buffer for every re-plan would race
        # with a copy the GPU has not yet reached.)
        self.plan_host = t.empty(nbytes, dtype=t.uint8, pin_memory=True)
        self.plan_dev = t.empty(nbytes, dtype=t.uint8, device=_lib.device())
        _lib.call("jx_batch_plan", arr, n, ctypes.c_void_p(self.plan_host.data_ptr()), nbytes)
        self.plan_dev.copy_(self.plan_host, non_blocking=True)
        self.groups = _lib.load().jx_batch_groups(ctypes.c_void_p(self.plan_host.data_ptr()))
        self.graph = None

    def enqueue_step(self):
        """Enqueue one cycle of every solve on the current stream."""
        _lib.call("jx_batch_step", ctypes.c_void_p(self.plan_host.data_ptr()),
                  ctypes.c_void_p(self.plan_dev.data_ptr()), self.blocks_per_sm, _lib.stream_handle())

    def capture(self, steps):
        """Capture `steps` cycles in a CUDA graph (call after one eager step)."""
        t = _lib.torch()
        t.cuda.synchronize()
        graph = t.cuda.CUDAGraph()
        with t.cuda.graph(graph):
            for _ in range(steps):
                self.enqueue_step()
        self.graph, self.graph_steps = graph, steps

    def states(self):
        if self.clocks is not None:
            return self.clocks.read()
        return [s.state() for s in self.solves]

    def run(self, steps_per_sync=16, use_graph=True):
        """Advance until every solve reached its tlim or nlim; returns the clocks."""
        self.enqueue_step()
        if all(c.done for c in self.states()):
            return self.states()
        if use_graph and self.graph is None:
            self.capture(steps_per_sync)
        while True:
            if use_graph:
                self.graph.replay()
            else:
                for _ in range(steps_per_sync):
                    self.enqueue_step()
            clocks = self.states()
            if all(c.done for c in clocks):
                return clocks
