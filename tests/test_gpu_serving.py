"""Serving form: continuous batching keeps each world's result independent of the mix."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_world_same_alone_and_in_the_mix(precision):
    from physkit_gb300.serve import StepServer

    def target_records(srv):
        return srv.templates.records(np.random.Generator(np.random.PCG64(11)), 200, 0)

    # the world under test, alone: 40 steps back to back
    alone = StepServer(max_worlds=8, max_bodies=20000, precision=precision)
    alone.open(0, 200, 1000, 0.0, records=target_records(alone))
    alone.admit(0.0)
    wid = next(iter(alone.live))
    for _ in range(40):
        alone.advance(wid, 0.0)
        alone.step_once()
    a = alone.world_state(wid)

    # the same world in a mix: other worlds come and go, and it sits out random batched steps
    rng = np.random.Generator(np.random.PCG64(3))
    mix = StepServer(max_worlds=8, max_bodies=20000, precision=precision)
    for k in range(3):
        mix.open(100 + k, int(rng.integers(50, 300)), 25, 0.0)
    mix.admit(0.0)
    mix.open(0, 200, 1000, 0.0, records=target_records(mix))
    (_, target), = mix.admit(0.0)
    done = 0
    while done < 40:
        for lw in list(mix.live.values()):
            if lw.wid != target and rng.random() < 0.7:
                mix.advance(lw.wid, 0.0)
        if rng.random() < 0.6:
            mix.advance(target, 0.0)
            done += 1
        if len(mix.live) < 4 and rng.random() < 0.3:
            mix.open(200 + done, int(rng.integers(20, 200)), 10, 0.0)
            mix.admit(0.0)
        mix.step_once()
    while mix.live[target].pending:
        mix.step_once()
    assert mix.live[target].steps_done == 40
    assert mix.steps > 40  # the target sat out some of the batched steps
    b = mix.world_state(target)
    assert np.array_equal(b[:, :13], a[:, :13])
    alone.close()
    mix.close()


def test_poisson_load_report_small():
    from physkit_gb300.serve import run_served

    rep = run_served(rate=2000, duration=0.5, warm_live=16, max_worlds=64, max_bodies=200_000, nmax=512, lanes=1)
    assert rep["completed_steps"] > 0 and rep["p99_ms"] is not None
    assert rep["p50_ms"] <= rep["p99_ms"] <= rep["p999_ms"]


def test_poisson_load_report_two_lanes():
    from physkit_gb300.serve import run_served

    rep = run_served(rate=2000, duration=0.5, warm_live=16, max_worlds=64, max_bodies=300_000, nmax=2048, lanes=2)
    assert rep["completed_steps"] > 0 and rep["p99_ms"] is not None and rep["lanes"] == 2
    assert rep["p50_ms"] <= rep["p99_ms"] <= rep["p999_ms"]
