"""Device-to-host copies into page-locked memory from lfg_host_alloc
(lfg_memcpy_d2h, lfg_coo_download): at 1 MB and more with 16-byte aligned
ends a copy kernel stores through the mapping, otherwise cudaMemcpyAsync;
both give the device bytes exactly, at any offset inside the allocation, and
never touch bytes outside the copied range."""
import numpy as np
import pytest

from parity import L, W, Run

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nbytes", [16, 4096, (1 << 20), (1 << 20) + 16, 3 * (1 << 20) + 7, 64 << 20])
@pytest.mark.parametrize("offset", [0, 16, 3])
def test_d2h_into_pinned(ctx, nbytes, offset):
    rng = np.random.default_rng(nbytes + offset)
    data = rng.integers(0, 256, nbytes, dtype=np.uint8)
    dev = ctx.to_device(data)
    pin = ctx.pinned((nbytes + 64,), np.uint8)
    pin.array[:] = 0xA5
    dst = pin.ptr.value + offset
    ctx.check(L.lib().lfg_memcpy_d2h(ctx.h, dst, dev.ptr, nbytes))
    got = pin.array[offset:offset + nbytes]
    assert np.array_equal(got, data)
    assert (pin.array[:offset] == 0xA5).all() and (pin.array[offset + nbytes:] == 0xA5).all()
    # pageable destination: the copy engines
    host = np.zeros(nbytes, np.uint8)
    ctx.check(L.lib().lfg_memcpy_d2h(ctx.h, host.ctypes.data, dev.ptr, nbytes))
    assert np.array_equal(host, data)


def test_coo_download_into_pinned(ctx):
    r = Run(ctx, W.config2(40))
    coo = r.gpu_matrix()
    ref = coo.triplets()
    pin = ctx.pinned((len(ref) + 2,), L.TRIPLET_DTYPE)
    coo.download_into(pin)
    assert np.array_equal(pin.array[:len(ref)], ref)
