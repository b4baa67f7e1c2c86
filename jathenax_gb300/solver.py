"""A device-resident solve: state, scratch, workspace, clock and forcing tables.

One :class:`Solve` is one ``evolve_isothermal`` run (run.py:20-69). Its
state lives in HBM for the whole run; every cycle is enqueued as one
``jx_step`` (begin-step/dt, optional render, the fused stages, optional kick)
and the host only reads the 128-byte clock back every ``steps_per_sync``
cycles to learn whether tlim or nlim was reached. Runs without an SGS hook
replay a CUDA graph of ``steps_per_sync`` captured cycles.
"""

import ctypes
import json

import numpy as np

from . import _lib
from .hydro import RK_STAGES, _Forcing, make_desc, run_stages


class Solve:
    """Device-resident evolve_isothermal run."""

    def __init__(self, U, dx, dy, cs, dfloor, integrator, cfl, tlim, nlim, *,
                 viscosity=0.0, smagorinsky_cs=0.0, drag_rate=0.0, forcing=None,
                 dt_update=1.0, tdriv_start=0.0, dedt=0.0, reconstruct="ppm4", rsolver="roe",
                 predict_stress=None, sgs_weights=None, tile=(0, 0), dtype=None, clock=None):
        t = _lib.torch()
        RK_STAGES[integrator]
        U_dev = _lib.to_device(U, dtype)
        self.desc = make_desc(U_dev.shape, U_dev.dtype, dx, dy, cs, dfloor, integrator,
                              viscosity=viscosity, smagorinsky_cs=smagorinsky_cs,
                              drag_rate=drag_rate, reconstruct=reconstruct, rsolver=rsolver,
                              tile=tile)
        # The solve owns its state: copy a caller's device array, adopt a fresh one.
        self.S = U_dev.clone() if U_dev is U else U_dev
        self.A = t.empty_like(self.S)
        self.B = t.empty_like(self.S)
        self.ws, self.nbytes = _lib.workspace(self.desc)
        self.predict_stress, self.sgs_weights = predict_stress, sgs_weights
        self.forcing = None
        n_updates = 0
        if forcing is not None:
            from .forcing import _device_tables
            coefficients, basis = forcing
            tables = _device_tables(coefficients, basis, self.S.dtype)
            if tables[1].shape[1] != self.S.shape[1] or tables[3].shape[1] != self.S.shape[0]:
                raise ValueError("forcing basis does not match the grid")
            raw = t.zeros(tuple(self.S.shape[:2]) + (2,), dtype=self.S.dtype, device=self.S.device)
            self.forcing = _Forcing(raw, tables)
            n_updates = tables[0].shape[0]
        fresh = _lib.new_clock(
            tlim=float(tlim), nlim=int(nlim), cfl=float(cfl), t_start=float(tdriv_start),
            dt_update=float(dt_update), dedt=float(dedt), n_updates=n_updates)
        if clock is None:
            self.clock = fresh
        else:  # a 128-byte slice of a caller's buffer (batches read all clocks at once)
            if clock.numel() != 128 or clock.dtype != t.uint8:
                raise ValueError("clock storage must be 128 uint8 elements")
            clock.copy_(fresh)
            self.clock = clock
        self._idle_clock = None  # made on first capture
        self.graph = None
        self.graph_steps = 0
        _lib.call("jx_cfl_partials", ctypes.byref(self.desc), _lib.ptr(self.S), _lib.ptr(self.ws),
                  self.nbytes, _lib.stream_handle())

    def set_tile(self, tile):
        """Switch the stage tile (see make_desc's ``tile``) of a live solve.

        The workspace grows if the new tile needs more CFL partial slots, the
        partials are recomputed from the current state and any captured graph
        is dropped. Float32 results do not depend on the tile; float64 results
        agree across tiles to rounding.
        """
        self.desc.tile_x, self.desc.tile_y = int(tile[0]), int(tile[1])
        size = ctypes.c_size_t()
        _lib.call("jx_workspace_bytes", ctypes.byref(self.desc), ctypes.byref(size))
        if size.value > self.nbytes:
            self.ws, self.nbytes = _lib.workspace(self.desc)
        self.graph, self.graph_steps = None, 0
        _lib.call("jx_cfl_partials", ctypes.byref(self.desc), _lib.ptr(self.S), _lib.ptr(self.ws),
                  self.nbytes, _lib.stream_handle())

    # -- enqueueing -----------------------------------------------------------
    def enqueue_step(self, clock=None):
        """Enqueue one full cycle (no SGS hook) on the current stream."""
        clock = self.clock if clock is None else clock
        forcing = ctypes.byref(self.forcing.struct) if self.forcing is not None else None
        _lib.call("jx_step", ctypes.byref(self.desc), _lib.ptr(self.S), _lib.ptr(self.A),
                  _lib.ptr(self.B), forcing, _lib.ptr(clock), _lib.ptr(self.ws), self.nbytes,
                  _lib.stream_handle())

    def _hooked_step(self):
        """One cycle with the SGS predictor: stages are driven from the host."""
        stream = _lib.stream_handle()
        forced = self.forcing is not None
        _lib.call("jx_begin_step", ctypes.byref(self.desc), _lib.ptr(self.clock), int(forced),
                  _lib.ptr(self.ws), self.nbytes, stream)
        if _lib.read_clock(self.clock).done:
            return False
        if forced:
            _lib.call("jx_force_render", ctypes.byref(self.desc), ctypes.byref(self.forcing.struct),
                      _lib.ptr(self.clock), stream)
        run_stages(self.desc, self.S, clock=self.clock, ws=self.ws, nbytes=self.nbytes,
                   forcing=self.forcing, predict_stress=self.predict_stress,
                   sgs_weights=self.sgs_weights, out=self.A)
        self.S, self.A = self.A, self.S
        if self.desc.smagorinsky_cs > 0.0:
            _lib.call("jx_cfl_partials", ctypes.byref(self.desc), _lib.ptr(self.S),
                      _lib.ptr(self.ws), self.nbytes, stream)
        return True

    def capture(self, steps):
        """Capture `steps` cycles into a CUDA graph (after a launch on an idle clock)."""
        t = _lib.torch()
        if self._idle_clock is None:
            self._idle_clock = _lib.new_clock(done=1)
        self.enqueue_step(self._idle_clock)  # sets per-kernel attributes; changes nothing
        t.cuda.synchronize()
        graph = t.cuda.CUDAGraph()
        with t.cuda.graph(graph):
            for _ in range(steps):
                self.enqueue_step()
        self.graph, self.graph_steps = graph, steps

    # -- driving --------------------------------------------------------------
    def state(self):
        return _lib.read_clock(self.clock)

    def box_sums(self):
        """Float64 sums of every conserved component over the grid (run.py:186-187)."""
        t = _lib.torch()
        out = t.empty(self.desc.nvar, dtype=t.float64, device=self.S.device)
        _lib.call("jx_box_sums", ctypes.byref(self.desc), _lib.ptr(self.S), _lib.ptr(out),
                  _lib.ptr(self.ws), self.nbytes, _lib.stream_handle())
        return out.cpu().numpy()

    def as_jx_solve(self):
        """This solve as the C ABI's jx_solve (for batches)."""
        js = _lib.SolveStruct()
        js.desc = self.desc
        js.S, js.A, js.B = self.S.data_ptr(), self.A.data_ptr(), self.B.data_ptr()
        js.clock = self.clock.data_ptr()
        if self.forcing is not None:
            js.forcing = self.forcing.struct
        js.workspace = self.ws.data_ptr()
        js.workspace_bytes = self.nbytes
        return js

    def run(self, steps_per_sync=32, use_graph=True, checkpoint=None, checkpoint_every=0):
        """Advance until tlim or nlim; returns the final clock.

        With ``checkpoint`` (a path) the run is written there (see
        :meth:`checkpoint`) whenever ``checkpoint_every`` more cycles have
        completed (checked every ``steps_per_sync`` cycles) and at the end.
        """
        last = self.state().cycle
        if self.predict_stress is not None:
            while self._hooked_step():
                last = self._maybe_checkpoint(checkpoint, checkpoint_every, last)
        else:
            if use_graph and self.graph is None:
                self.capture(steps_per_sync)
            while True:
                if use_graph:
                    self.graph.replay()
                else:
                    for _ in range(steps_per_sync):
                        self.enqueue_step()
                if self.state().done:
                    break
                last = self._maybe_checkpoint(checkpoint, checkpoint_every, last)
        if checkpoint is not None:
            self.checkpoint(checkpoint)
        return self.state()

    def _maybe_checkpoint(self, path, every, last):
        if path is None or every <= 0:
            return last
        cycle = self.state().cycle
        if cycle - last >= every:
            self.checkpoint(path)
            return cycle
        return last

    def result(self):
        c = self.state()
        return self.S, c.time, c.prev_dt, c.cycle

    # -- checkpoint / resume ----------------------------------------------------
    def _desc_fields(self):
        return {name: getattr(self.desc, name) for name, _ in self.desc._fields_}

    def checkpoint(self, path):
        """Write the resident run to an npz file for an exact resume.

        Keys: ``conserved``, ``time``, ``dt`` and ``cycle`` as in the
        reference's output (run.py:184-185), plus what an exact resume needs:
        ``clock`` (the 128-byte device clock), ``workspace`` (the CFL partials
        the next dt is chosen from, the forcing sums), ``raw_force`` (the
        cached forcing field of a forced run) and ``desc`` (the problem
        description, checked on resume).
        """
        c = self.state()
        arrays = dict(conserved=self.S.cpu().numpy(), time=np.float64(c.time), dt=np.float64(c.prev_dt),
                      cycle=np.int32(c.cycle), clock=self.clock.cpu().numpy(),
                      workspace=self.ws.cpu().numpy(), desc=np.array(json.dumps(self._desc_fields())))
        if self.forcing is not None:
            arrays["raw_force"] = self.forcing.raw.cpu().numpy()
        np.savez(path, **arrays)

    def resume(self, path):
        """Continue from a checkpoint written by a Solve built with the same
        arguments (the end time, cycle limit and forcing-table length may be
        larger); the continued run is bitwise the uninterrupted one."""
        t = _lib.torch()
        with np.load(path, allow_pickle=False) as data:
            if json.loads(str(data["desc"])) != self._desc_fields():
                raise ValueError("checkpoint was written for a different problem description")
            U = data["conserved"]
            if tuple(U.shape) != tuple(self.S.shape) or U.dtype != np.dtype(str(self.S.dtype)[6:]):
                raise ValueError("checkpoint state does not match this solve's shape and precision")
            if ("raw_force" in data) != (self.forcing is not None):
                raise ValueError("checkpoint and solve disagree about forcing")
            if data["workspace"].size != self.nbytes or data["clock"].size != 128:
                raise ValueError("checkpoint workspace or clock has the wrong size")
            # The saved clock carries time, cycle, dt history and the forcing
            # schedule; the limits are this solve's, and begin-step re-tests them.
            mine = self.state()
            c = _lib.Clock.from_buffer_copy(data["clock"].tobytes())
            c.tlim, c.nlim, c.n_updates, c.done = mine.tlim, mine.nlim, mine.n_updates, 0
            self.S.copy_(t.from_numpy(U))
            self.clock.copy_(t.from_numpy(np.frombuffer(bytes(c), dtype=np.uint8).copy()))
            self.ws.copy_(t.from_numpy(data["workspace"]))
            if self.forcing is not None:
                self.forcing.raw.copy_(t.from_numpy(data["raw_force"]))

    def advance_host(self, U_host, out_host, steps=1):
        """Load U from host memory, advance `steps` cycles, write the state back.

        U_host/out_host are CPU tensors of the state's shape and dtype (pinned
        memory makes both copies asynchronous). The CFL partials are
        recomputed from the loaded state, as evolve_isothermal does at its
        start. Nothing is synchronised here; the caller synchronises.
        """
        self.S.copy_(U_host, non_blocking=True)
        _lib.call("jx_cfl_partials", ctypes.byref(self.desc), _lib.ptr(self.S), _lib.ptr(self.ws),
                  self.nbytes, _lib.stream_handle())
        for _ in range(steps):
            self.enqueue_step()
        out_host.copy_(self.S, non_blocking=True)

    def advance_host_many(self, inputs, outputs, steps=1):
        """advance_host over a sequence of independent host states, with each
        state's upload and download overlapping the cycles of its neighbours.

        inputs/outputs are sequences of pinned CPU tensors of the state's shape
        and dtype. State k is uploaded into one of three device buffers (so the
        upload of state k+1 and the download of state k-1 run at the same
        time) on an upload stream, advanced on the current stream (CFL partials from the
        loaded state, then `steps` cycles, the clock and workspace shared as in
        advance_host, so results equal calling advance_host on each state in
        turn) and downloaded on a download stream. The current stream waits for
        the last download; nothing is synchronised with the host.
        """
        t = _lib.torch()
        if getattr(self, "_host_bufs", None) is None:
            self._host_bufs = tuple(t.empty_like(self.S) for _ in range(3))
            self._up, self._down = t.cuda.Stream(), t.cuda.Stream()
        cur = t.cuda.current_stream()
        nbuf = len(self._host_bufs)
        free = [None] * nbuf  # download of the buffer's previous state has finished
        forcing = ctypes.byref(self.forcing.struct) if self.forcing is not None else None
        handle = _lib.stream_handle()
        for k, (U_host, out_host) in enumerate(zip(inputs, outputs)):
            b = k % nbuf
            buf = self._host_bufs[b]
            if k == 0:
                self._up.wait_stream(cur)  # earlier work on the buffers is ordered first
            if free[b] is not None:
                self._up.wait_event(free[b])
            with t.cuda.stream(self._up):
                buf.copy_(U_host, non_blocking=True)
            loaded = t.cuda.Event()
            loaded.record(self._up)
            cur.wait_event(loaded)
            _lib.call("jx_cfl_partials", ctypes.byref(self.desc), _lib.ptr(buf), _lib.ptr(self.ws),
                      self.nbytes, handle)
            for _ in range(steps):
                _lib.call("jx_step", ctypes.byref(self.desc), _lib.ptr(buf), _lib.ptr(self.A), _lib.ptr(self.B),
                          forcing, _lib.ptr(self.clock), _lib.ptr(self.ws), self.nbytes, handle)
            stepped = t.cuda.Event()
            stepped.record(cur)
            self._down.wait_event(stepped)
            with t.cuda.stream(self._down):
                out_host.copy_(buf, non_blocking=True)
            free[b] = t.cuda.Event()
            free[b].record(self._down)
        for event in free:
            if event is not None:
                cur.wait_event(event)

    def enqueue_stage(self, stage, U_in, V_in, U_out, V_out=None):
        """Enqueue one fused stage kernel alone (used to time the kernel in isolation)."""
        _lib.call("jx_stage", ctypes.byref(self.desc), int(stage), _lib.ptr(U_in), _lib.ptr(V_in),
                  _lib.ptr(U_out), _lib.ptr(V_out), None, 0, _lib.ptr(self.clock), None,
                  _lib.ptr(self.ws), self.nbytes, _lib.stream_handle())

    def set_clock(self, **fields):
        """Overwrite clock fields from the host (synchronous, small)."""
        c = self.state()
        for key, value in fields.items():
            setattr(c, key, value)
        host = np.frombuffer(bytes(c), dtype=np.uint8).copy()
        self.clock.copy_(_lib.torch().from_numpy(host))


def check_evolve_args(viscosity, smagorinsky_cs, drag_rate, dedt, forcing, dt_update, tdriv_start):
    """Argument checks of run.py:29-34."""
    from math import isfinite
    for name, value in (("viscosity", viscosity), ("smagorinsky_cs", smagorinsky_cs),
                        ("drag_rate", drag_rate), ("dedt", dedt)):
        if not isfinite(value) or value < 0.0:
            raise ValueError(f"{name} must be finite and nonnegative")
    if forcing is not None and (not 0.0 < dt_update < np.inf or not isfinite(tdriv_start)):
        raise ValueError("dt_update must be finite and positive and tdriv_start finite")
