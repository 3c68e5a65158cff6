"""Failure detection on the GPU without faulting it.

* A bounded wait that runs out (on a barrier nothing arrives on, limit 2000
  iterations) makes the kernel record a timeout in the box state, wait for
  its own TMA copies, and return; the host reads the status, and the same
  context keeps working.
* A NaN planted in the host f-array before upload gives a non-finite CFL
  timestep, which the kernel flags instead of propagating silently."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _box(pc, ic, **kw):
    p = pc.default_params(nx=32, ny=32, nz=32, gamma=1.0, nu=5e-3, eta=5e-3, dt=5e-3, precision=8)
    p.update(**kw)
    f = ic.zeros(p)
    ic.gaussian_noise(f, p, ["ux", "uy", "uz", "ax", "ay", "az"], 1e-3, 3)
    b = pc.Box(p)
    b.load(f)
    return b, f


def test_bounded_wait_timeout_is_reported_and_recoverable(pc, ic):
    L = pc.load()
    b, f = _box(pc, ic)
    try:
        L.pcgb_set_wait_limit(2000)
        L.pcgb_inject_wait_failure(1)
        b.steps(1)
        with pytest.raises(pc.PcgbError, match="bounded device wait"):
            b.sync()
    finally:
        L.pcgb_inject_wait_failure(0)
        L.pcgb_set_wait_limit(0)
        L.pcgb_clear_error()
    # the context is usable: reload and step normally
    b.load(f)
    b.steps(2)
    b.sync()
    g = b.store()
    assert np.all(np.isfinite(g))


def test_nan_in_host_state_is_flagged(pc, ic):
    L = pc.load()
    b, f = _box(pc, ic, dt=0.0, dt_mode=1)
    f[10, 10, 10, 0] = np.nan
    b.load(f)
    b.steps(1)
    with pytest.raises(pc.PcgbError, match="non-finite"):
        b.sync()
    L.pcgb_clear_error()


@pytest.mark.parametrize("tile", [5, 7])
def test_bounded_wait_timeout_tensor_memory_tile(pc, ic, tile):
    """The same timeout path in the FP32 pair kernels that hold tensor memory (8 and 12
    warps): the CTAs leave their tiles, release their tensor memory and return; the next
    launches allocate it again and the box steps normally after a reload."""
    L = pc.load()
    b, f = _box(pc, ic, precision=4, comp=1, tile=tile)
    try:
        L.pcgb_set_wait_limit(2000)
        L.pcgb_inject_wait_failure(1)
        b.steps(1)
        with pytest.raises(pc.PcgbError, match="bounded device wait"):
            b.sync()
    finally:
        L.pcgb_inject_wait_failure(0)
        L.pcgb_set_wait_limit(0)
        L.pcgb_clear_error()
    b.load(f)
    b.steps(2)
    b.sync()
    assert np.all(np.isfinite(b.store()))
