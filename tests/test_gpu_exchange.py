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
