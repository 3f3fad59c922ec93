"""gbh_exchange_bodies: one call returns the current bodies and installs new
ones (the two copies overlapped in chunks); stepping after it equals stepping
after a plain upload of the same bodies."""
import numpy as np
import pytest

from gravity_gb300 import BarnesHut, abi, ic

pytestmark = pytest.mark.gpu


def test_exchange_returns_state_and_installs_input(gbh_lib):
    torch = pytest.importorskip("torch")
    n = 100003  # chunks of uneven length
    a = ic.plummer(n, seed=1)
    b = ic.plummer(n, seed=2)
    p = abi.step_params(theta=0.5, softening=1e-4)
    sim = BarnesHut(n, ic.exact_bounds(a), abi.units(G=1.0))
    sim.upload_bodies(a)
    sim.init()
    sim.step(p)
    want_state = sim.read_bodies()
    pin = torch.empty(n * abi.BODY_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(abi.BODY_DTYPE)
    sim.exchange_bodies(pin, b)
    assert np.array_equal(pin.view(np.uint32), want_state.view(np.uint32))
    assert np.array_equal(sim.read_bodies().view(np.uint32), b.view(np.uint32))
    # the next step sees exactly the installed bodies
    sim.step(p)
    ref = BarnesHut(n, ic.exact_bounds(a), abi.units(G=1.0))
    ref.upload_bodies(a)
    ref.init()
    ref.step(p)
    ref.upload_bodies(b)
    ref.step(p)
    assert np.array_equal(sim.read_bodies().view(np.uint32), ref.read_bodies().view(np.uint32))
    # a sub-range, from pageable memory
    out = np.zeros(1000, abi.BODY_DTYPE)
    sim.exchange_bodies(out, a[5000:6000], offset=5000)
    assert np.array_equal(sim.read_bodies()[5000:6000].view(np.uint32), a[5000:6000].view(np.uint32))


def _pinned(torch, n):
    return torch.empty(n * abi.BODY_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(abi.BODY_DTYPE)


def test_streamed_steps_equal_upload_step_read(gbh_lib):
    # every call installs a new state and returns the previous call's result:
    # the results must be bit-identical to upload + step + read per state
    torch = pytest.importorskip("torch")
    # (8 calls: the three body buffers rotate, so every pairing of input and
    # output buffers and both parities come round)
    n = 70001
    calls = 8
    states = [ic.plummer(n, seed=10 + k) for k in range(calls + 1)]
    bounds = ic.exact_bounds(states[0])
    p = abi.step_params(theta=0.5, softening=1e-4, bounds=abi.BOUNDS_DYNAMIC)
    ref = BarnesHut(n, bounds, abi.units(G=1.0))
    ref.upload_bodies(states[0])
    ref.init()
    want = []
    for k in range(calls):
        ref.upload_bodies(states[k])
        ref.step(p)
        want.append(ref.read_bodies())
    sim = BarnesHut(n, bounds, abi.units(G=1.0))
    sim.upload_bodies(states[0])
    sim.init()
    nxt, out = _pinned(torch, n), _pinned(torch, n)
    got = []
    for k in range(calls):
        nxt[:] = states[k + 1]
        out.fill(0)
        sim.step_streamed(p, nxt, out)
        if k:
            got.append(out.copy())
    sim.step_streamed_finish(out)
    got.append(out.copy())
    for k in range(calls):
        assert np.array_equal(got[k].view(np.uint32), want[k].view(np.uint32)), k
    # the last installed input is the current state
    assert np.array_equal(sim.read_bodies().view(np.uint32), states[calls].view(np.uint32))


def test_streamed_steps_mixed_with_other_calls(gbh_lib):
    # a pending result survives plain steps and uploads between streamed
    # calls, with and without a next input
    torch = pytest.importorskip("torch")
    n = 60001
    s = [ic.plummer(n, seed=30 + k) for k in range(5)]
    bounds = ic.exact_bounds(s[0])
    p = abi.step_params(theta=0.5, softening=1e-4, bounds=abi.BOUNDS_DYNAMIC)
    ref = BarnesHut(n, bounds, abi.units(G=1.0))
    ref.upload_bodies(s[0])
    ref.init()

    def run(state, steps):
        ref.upload_bodies(state)
        for _ in range(steps):
            ref.step(p)
        return ref.read_bodies()

    r0 = run(s[0], 1)
    r1 = run(s[1], 1)
    r2 = run(r1, 2)
    r3 = run(s[3], 1)
    sim = BarnesHut(n, bounds, abi.units(G=1.0))
    sim.upload_bodies(s[0])
    sim.init()
    pin, out = _pinned(torch, n), _pinned(torch, n)
    pin[:] = s[1]
    sim.step_streamed(p, pin, None)          # steps s0, installs s1
    sim.step_streamed(p, None, out)          # returns r0, steps s1 (r1 stays the state)
    assert np.array_equal(out.view(np.uint32), r0.view(np.uint32))
    sim.step(p)                              # a plain step on r1
    pin[:] = s[2]
    sim.step_streamed(p, pin, out)           # returns r1, steps again, installs s2
    assert np.array_equal(out.view(np.uint32), r1.view(np.uint32))
    sim.upload_bodies(s[3])                  # replaces s2
    pin[:] = s[4]
    sim.step_streamed(p, pin, out)           # returns r2, steps s3, installs s4
    assert np.array_equal(out.view(np.uint32), r2.view(np.uint32))
    sim.step_streamed_finish(out)
    assert np.array_equal(out.view(np.uint32), r3.view(np.uint32))
    assert np.array_equal(sim.read_bodies().view(np.uint32), s[4].view(np.uint32))
    sim.step(p)
    assert np.array_equal(sim.read_bodies().view(np.uint32), run(s[4], 1).view(np.uint32))


def test_streamed_steps_without_input_record_the_trajectory(gbh_lib):
    # next_input NULL: a plain simulation whose every state comes back
    torch = pytest.importorskip("torch")
    n = 50000
    b = ic.plummer(n, seed=4)
    p = abi.step_params(theta=0.5, softening=1e-4)
    a = BarnesHut(n, ic.exact_bounds(b), abi.units(G=1.0))
    c = BarnesHut(n, ic.exact_bounds(b), abi.units(G=1.0))
    for x in (a, c):
        x.upload_bodies(b)
        x.init()
    out = _pinned(torch, n)
    traj = []
    for k in range(4):
        a.step_streamed(p, None, out if k else None)
        if k:
            traj.append(out.copy())
    a.step_streamed_finish(out)
    traj.append(out.copy())
    for k in range(4):
        c.step(p)
        assert np.array_equal(traj[k].view(np.uint32), c.read_bodies().view(np.uint32)), k
    assert np.array_equal(a.read_bodies().view(np.uint32), c.read_bodies().view(np.uint32))
