"""Serving: continuous batching admits requests by HBM budget; every result
equals the same request run alone, bitwise."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_stream(n=10, seed=3, rate=400.0):
    from jathenax_gb300.serve import make_stream
    return make_stream(n, rate, seed=seed, side_range=(24, 96), tlim_range=(0.005, 0.03),
                       fp32_fraction=0.6)


def test_each_served_result_equals_the_request_run_alone():
    from jathenax_gb300.serve import Server, build_solve
    reqs = small_stream()
    assert len({r.problem for r in reqs}) >= 2 and len({r.dtype for r in reqs}) == 2
    stats = Server(budget_bytes=1e9, tile=(32, 16), steps_per_tick=3, keep_results=True).run(reqs)
    assert stats["requests"] == len(reqs) and stats["peak_live"] >= 2
    assert 0 < stats["tts_p50_s"] <= stats["tts_p99_s"]
    for r in reqs:
        alone = build_solve(r, dtype=r.served_dtype)
        alone.run(steps_per_sync=4)
        np.testing.assert_array_equal(r.result, alone.S.cpu().numpy(), err_msg=str(r))
        assert r.cycles == alone.state().cycle


def test_admission_holds_live_memory_under_the_budget():
    from jathenax_gb300.serve import Server, footprint_bytes
    reqs = small_stream(8, seed=5)
    budget = 2.2 * max(footprint_bytes(r) for r in reqs)
    stats = Server(budget_bytes=budget, tile=(32, 16), steps_per_tick=2).run(reqs)
    assert stats["requests"] == 8
    assert 0 < stats["peak_bytes"] <= budget
    assert stats["peak_live"] < 8
    assert all(r.finished >= r.admitted >= r.arrival for r in reqs)


def test_a_failing_request_is_retired_and_the_others_complete():
    """Host-side fault injection: one request starts with a NaN in its state."""
    from jathenax_gb300.serve import Server, build_solve
    reqs = small_stream(6, seed=11)
    victim = reqs[2].rid

    def builder(req, tile, clock=None, dtype=None):
        solve = build_solve(req, tile, clock=clock, dtype=dtype)
        if req.rid == victim:
            solve.S[solve.S.shape[0] // 2, solve.S.shape[1] // 2, 1] = float("nan")
        return solve

    stats = Server(budget_bytes=1e9, tile=(32, 16), steps_per_tick=2, builder=builder).run(reqs)
    assert stats["failed"] == 1 and stats["completed"] == 5
    assert reqs[2].error is not None and "non-finite" in reqs[2].error
    assert all(r.error is None for r in reqs if r.rid != victim)


def test_replanning_every_tick_keeps_results_exact():
    """Many short requests and one step per tick: the batch is re-planned at
    almost every tick while earlier ticks are still queued on the GPU."""
    from jathenax_gb300.serve import Server, build_solve, make_stream
    reqs = make_stream(24, 2000.0, seed=8, side_range=(16, 64), tlim_range=(0.05, 0.3), fp32_fraction=0.7)
    for _ in range(2):
        for r in reqs:
            r.admitted = r.finished = r.result = None
        stats = Server(budget_bytes=1e9, tile=(32, 16), steps_per_tick=1, keep_results=True).run(reqs)
        assert stats["completed"] == len(reqs) and stats["ticks"] > len(reqs)
    for r in reqs:
        alone = build_solve(r, dtype=r.served_dtype)
        alone.run(steps_per_sync=4)
        np.testing.assert_array_equal(r.result, alone.S.cpu().numpy(), err_msg=str(r))


def test_warmup_touches_every_method_and_precision():
    from jathenax_gb300.serve import Server, warmup_requests
    reqs = warmup_requests()
    assert len(reqs) == 2 * 3 * 5 * 3
    stats = Server(budget_bytes=1e9, tile=(32, 16)).run(reqs)
    assert stats["completed"] == len(reqs)


def test_tuned_tiles_per_size_class_keep_results_exact():
    """Automatic tiles: each request runs on its (precision, size class,
    reconstruction) tile from the autotuner, and equals the same request run
    alone on that tile."""
    from jathenax_gb300.serve import Server, build_solve, make_stream, size_class
    reqs = make_stream(12, 600.0, seed=21, side_range=(40, 300), tlim_range=(0.01, 0.04), fp32_fraction=0.6)
    server = Server(budget_bytes=2e9, steps_per_tick=4, keep_results=True)
    stats = server.run(reqs)
    assert stats["completed"] == len(reqs)
    assert len({size_class(r.side) for r in reqs}) >= 2
    table = server.tile_table()
    assert table and all(set(v["knobs"]) == {"staging", "columns_per_lane", "rows", "blocks_per_sm"}
                         for v in table.values())
    for r in reqs:
        alone = build_solve(r, server.tile_for(r), dtype=r.served_dtype)
        alone.run(steps_per_sync=4)
        np.testing.assert_array_equal(r.result, alone.S.cpu().numpy(), err_msg=str(r))


def test_guarded_float32_results_stay_within_1e5_of_float64():
    """A mixed stream with the precision guard on: every request served in
    float32 is within 1e-5 (L1 density, relative) of the same request run in
    float64, and the at-risk ones were promoted."""
    from jathenax_gb300.diagnostics import relative_l1
    from jathenax_gb300.serve import FP32_ERR_BAR, Server, build_solve, fp32_error_estimate, make_stream
    reqs = make_stream(30, 800.0, seed=33, side_range=(64, 160), tlim_range=(0.1, 1.2), fp32_fraction=1.0)
    stats = Server(budget_bytes=4e9, tile=(32, 16), steps_per_tick=8, keep_results=True).run(reqs)
    assert stats["completed"] == len(reqs)
    estimates = [fp32_error_estimate(r.problem, r.reconstruct, r.side, r.tlim) for r in reqs]
    at_risk = [r for r, e in zip(reqs, estimates) if e is None or e > FP32_ERR_BAR]
    assert at_risk and all(r.served_dtype == "float64" for r in at_risk)
    assert stats["promoted_to_float64"] == len(at_risk)
    served32 = [r for r in reqs if r.served_dtype == "float32"]
    assert len(served32) >= len(reqs) // 2
    for r in served32:
        ref = build_solve(r, dtype="float64")
        ref.run(steps_per_sync=16)
        err = float(relative_l1(r.result, ref.S.cpu().numpy())[0])
        assert err <= 1e-5, (str(r), err)
