"""Row-slab parallel driver of the float64 oracle on host cores.

TEST INFRASTRUCTURE ONLY: the CPU-baseline leg of ``bench.py`` (our line's
``cpu_baseline`` and the ``--impl reference`` arm) and ``tests/`` use it; the
shipped package never does.

It runs the oracle's evolve cycle - the CFL timestep (``hydro_oracle.timestep``,
hydro.py:63-89) followed by ``hydro_oracle.step``'s stage loop (hydro.py:92-146)
- on one n x n periodic grid split into row slabs, one ``spawn``ed process
per slab, so that the reference algorithm's CPU rate is measured on the same
grid as the GPU line instead of on small independent samples. Each stage a
process reads its rows plus GHOST rows on either side from a shared state
buffer (double-buffered, one barrier per stage), computes the primitives,
the face states, fluxes and divergence of its own rows, and combines them
with its own rows of the RK registers. Every operation of the inviscid stage
is per cell or a periodic neighbour access within 3 rows, and the CFL
minimum is reduced exactly (a minimum of minima), so the result is bit for
bit ``hydro_oracle.step`` on the whole grid (tests/test_oracle_slab.py).
Viscosity, Smagorinsky stress, drag, forcing and the SGS hook are not
supported here (the throughput workload has none of them).
"""

import os
import tempfile
import time

import numpy as np

from oracle import hydro_oracle as H

# Rows of the neighbours a stage needs: a y-face state reads cells j-3..j+2
# (the edges of the two cells beside the face, each from faces that span
# two cells either side), and the divergence reads the faces j and j+1.
GHOST = 3
# A worker that waits longer than this at a barrier gives up (another one died).
BARRIER_TIMEOUT_S = 600.0


def slab_bounds(n, procs, rank):
    """Rows [r0, r1) of slab `rank` of `procs` over n rows."""
    return rank * n // procs, (rank + 1) * n // procs


def _stage_rhs(U_pad, h, dx, dy, cs, dfloor, recon, solver):
    """Divergence of the h own rows from the padded slab (GHOST rows either side)."""
    _, W_pad = H.primitives(U_pad, dfloor)
    own = W_pad[GHOST:GHOST + h]
    lx, rx = H.face_states(own, 1, recon, dfloor)
    fx = H.face_flux(lx, rx, cs, 1, solver)
    ly, ry = H.face_states(W_pad, 0, recon, dfloor)
    fy = H.face_flux(ly, ry, cs, 0, solver)
    # hydro_oracle.divergence on the own rows, in its operation order.
    return (np.roll(fx, -1, axis=1) - fx) / dx + (fy[GHOST + 1:GHOST + 1 + h] - fy[GHOST:GHOST + h]) / dy


def _worker(rank, procs, path, shape, cycles, warm, params, barrier, mins_path):
    n, _, nv = shape
    dx = dy = 1.0 / n
    cs, dfloor, cfl, recon, solver, integrator = (params[k] for k in
                                                  ("cs", "dfloor", "cfl", "recon", "solver", "integrator"))
    buf = np.memmap(path, dtype=np.float64, mode="r+", shape=(2,) + shape)
    mins = np.memmap(mins_path, dtype=np.float64, mode="r+", shape=(2, procs))
    r0, r1 = slab_bounds(n, procs, rank)
    h = r1 - r0
    rows = np.arange(r0 - GHOST, r1 + GHOST) % n
    table = H.RK_TABLE[integrator]
    U = np.array(buf[0, r0:r1])
    cur, prev_dt, parity = 0, np.inf, 0
    t0 = None
    for cycle in range(warm + cycles):
        if cycle == warm:
            barrier.wait(BARRIER_TIMEOUT_S)
            t0 = time.perf_counter()
        # CFL timestep (the end-time clip never applies: no end time): this
        # slab's minimum, then the minimum over slabs.
        _, W = H.primitives(U, dfloor)
        mins[parity, rank] = min(np.min(dx / (np.abs(W[..., 1]) + cs)), np.min(dy / (np.abs(W[..., 2]) + cs)))
        barrier.wait(BARRIER_TIMEOUT_S)
        limit = np.min(mins[parity])
        parity ^= 1
        prev_dt = float(np.minimum(2.0 * prev_dt, cfl * limit))
        # hydro_oracle.step: floor, then the stages, each ending with a floor.
        U, _ = H.primitives(U, dfloor)
        V = U
        for coeffs in table:
            buf[cur, r0:r1] = U
            barrier.wait(BARRIER_TIMEOUT_S)
            div = _stage_rhs(np.asarray(buf[cur, rows]), h, dx, dy, cs, dfloor, recon, solver)
            U, V = H.rk_combine(U, V, div, prev_dt, coeffs)
            U, _ = H.primitives(U, dfloor)
            cur ^= 1
    elapsed = time.perf_counter() - t0
    buf[cur, r0:r1] = U
    buf.flush()
    barrier.wait(BARRIER_TIMEOUT_S)
    return cur, elapsed


def _entry(rank, procs, path, shape, cycles, warm, params, barrier, mins_path, results):
    """Process body: the worker's (rank, cur, seconds), or (rank, None, error text)."""
    try:
        cur, elapsed = _worker(rank, procs, path, shape, cycles, warm, params, barrier, mins_path)
        results.put((rank, cur, elapsed))
    except BaseException as exc:  # report, and release the others from the barrier
        barrier.abort()
        results.put((rank, None, f"{type(exc).__name__}: {exc}"))


def _scratch_dir(nbytes):
    """/dev/shm when it has room for the buffers, else the default temporary directory."""
    try:
        st = os.statvfs("/dev/shm")
        if st.f_bavail * st.f_frsize > 2 * nbytes:
            return "/dev/shm"
    except OSError:
        pass
    return None


def run(U0, cycles, procs=None, warm=0, cs=1.0, dfloor=1e-10, cfl=0.4, recon="ppm4", solver="roe",
        integrator="rk3"):
    """`warm` untimed then `cycles` timed evolve cycles of the oracle on the
    square periodic state U0 (n, n, nvar), in `procs` row slabs (default: one
    per host core). Returns (final state, seconds of the slowest process's
    timed cycles, processes used)."""
    import multiprocessing as mp
    import queue
    n = U0.shape[0]
    assert U0.shape[1] == n, "square grids only"
    assert cycles >= 1, "at least one timed cycle"
    procs = max(1, min(procs or os.cpu_count() or 1, n // GHOST))
    params = dict(cs=cs, dfloor=dfloor, cfl=cfl, recon=recon, solver=solver, integrator=integrator)
    tmp = tempfile.mkdtemp(prefix="jx_slab_", dir=_scratch_dir(2 * U0.nbytes))
    path, mins_path = os.path.join(tmp, "state"), os.path.join(tmp, "mins")
    workers = []
    try:
        buf = np.memmap(path, dtype=np.float64, mode="w+", shape=(2,) + U0.shape)
        buf[0] = U0
        buf.flush()
        np.memmap(mins_path, dtype=np.float64, mode="w+", shape=(2, procs)).flush()
        ctx = mp.get_context("spawn")  # the caller may hold a CUDA context
        barrier, results = ctx.Barrier(procs), ctx.Queue()
        workers = [ctx.Process(target=_entry, args=(r, procs, path, U0.shape, cycles, warm, params, barrier,
                                                    mins_path, results), daemon=True) for r in range(procs)]
        for w in workers:
            w.start()
        # A backstop only: a worker that dies is seen by its exit code, and one
        # left waiting at a barrier gives up after BARRIER_TIMEOUT_S and reports.
        got, deadline = {}, time.monotonic() + BARRIER_TIMEOUT_S * (warm + cycles + 2)
        while len(got) < procs:
            try:
                rank, cur, value = results.get(timeout=1.0)
            except queue.Empty:
                dead = [w.exitcode for w in workers if w.exitcode not in (None, 0)]
                if dead:
                    raise RuntimeError(f"an oracle slab worker exited with code {dead[0]}") from None
                if time.monotonic() > deadline:
                    raise RuntimeError("oracle slab workers stopped answering") from None
                continue
            if cur is None:
                raise RuntimeError(f"oracle slab worker {rank} failed: {value}")
            got[rank] = (cur, value)
        for w in workers:
            w.join()
        out = np.array(buf[got[0][0]])
        del buf
        return out, max(v for _, v in got.values()), procs
    finally:
        for w in workers:
            if w.is_alive():
                w.terminate()
                w.join()
        for f in (path, mins_path):
            if os.path.exists(f):
                os.remove(f)
        os.rmdir(tmp)
