"""Waiting on collision events through the C ABI (pk_world_wait / pk_world_dispatch) on the GPU,
against the oracle's event stream: the scenario of co_tests.cpp:383-430 (zero gravity, two unit boxes
approach at 1 m/s and pass through contact, a third box far away)."""
import numpy as np
import pytest

import pyoracle
from physkit_gb300 import scenes
from physkit_gb300.world import BODY_DTYPE, WAIT_COLLISION, WAIT_DESTROYED, WAIT_SEPARATION

pytestmark = pytest.mark.gpu


def _scene():
    b = np.zeros(3, dtype=BODY_DTYPE)
    b["shape"] = 0
    b["quat"][:, 0] = 1.0
    b["pos"] = [(-1, 0, 0), (1, 0, 0), (0, 10, 0)]
    b["vel"] = [(1, 0, 0), (-1, 0, 0), (0, 0, 0)]
    b["mass"] = 1.0
    b["inertia"][:, [0, 4, 8]] = 1.0
    b["restitution"] = 0.5
    b["friction"] = 0.5
    return scenes.Scene("co_tests two boxes", [("box", 1.0, 1.0, 1.0)], b, 1, (0.0, 0.0, 0.0))


def test_waiters_fire_on_the_oracles_event_steps():
    sc = _scene()
    world, h = scenes.make_world(sc, precision="f64")
    a, b, c = (int(x) for x in h)
    ow = pyoracle.OracleWorld(gravity=(0, 0, 0), iterations=sc.iterations, order="colour")
    pyoracle.load_scene(ow, sc)
    w_ab = world.wait(WAIT_COLLISION, a, b)
    w_sep = world.wait(WAIT_SEPARATION, b)
    w_c = world.wait(WAIT_COLLISION, c)
    w_cd = world.wait(WAIT_DESTROYED, c)
    w_cancel = world.wait(WAIT_COLLISION, a)
    world.cancel_wait(w_cancel)
    fired, oracle_first = {}, {}
    for step in range(1000):
        world.step(0.005)
        ow.step(0.005)
        for waiter, obj, other, kind, failed in world.dispatch():
            fired[waiter] = (step, obj, other, kind, failed)
        for key, kind in zip(*ow.events()):
            oracle_first.setdefault(int(kind), step)
    assert oracle_first.get(1) is not None and oracle_first.get(2) is not None
    assert fired[w_ab] == (oracle_first[1], a, b, WAIT_COLLISION, False)
    assert fired[w_sep] == (oracle_first[2], b, a, WAIT_SEPARATION, False)
    assert w_c not in fired and w_cd not in fired and w_cancel not in fired
    # removing c fails its collision waiter and fires its destruction waiter
    world.remove_rigid(c)
    got = {k[0]: k for k in world.dispatch()}
    assert got[w_c][3:] == (WAIT_COLLISION, True) and got[w_cd][3:] == (WAIT_DESTROYED, False)
    assert world.wait(WAIT_COLLISION, c) is None  # not alive: nothing to wait for
    world.close()
    ow.close()
