"""The random 32 B sector probe (midsx_gpu_probe_sectors) behind bench.py's L2 and HBM
ceilings: argument checks on the host (no device call), and on the GPU the exact count of its
atomic adds, all inside the buffer."""
import ctypes as C

import numpy as np
import pytest

from midsx_gb300 import native as N


def probe(ptr, nbytes, mode, requests, seed=1, stream=None):
    issued = C.c_uint64()
    st = N.load().midsx_gpu_probe_sectors(C.c_void_p(ptr), nbytes, mode, requests, seed, C.byref(issued),
                                          C.c_void_p(stream))
    return st, issued.value


@pytest.mark.parametrize("nbytes, mode, requests, ptr", [
    (1000, 0, 10, 4096),         # not a power of two
    (16, 0, 10, 4096),           # below one sector
    (1 << 20, 2, 10, 4096),      # unknown mode
    (1 << 20, 0, 0, 4096),       # no requests
    (1 << 20, 1, 10, 4100),      # unaligned buffer
    (1 << 20, 0, 10, 0),         # null buffer
])
def test_probe_rejects_bad_arguments_before_device_work(nbytes, mode, requests, ptr):
    st, issued = probe(ptr, nbytes, mode, requests)
    assert st == N.INVALID_ARG
    assert issued == 0


@pytest.mark.gpu
@pytest.mark.parametrize("mib", [1, 64])
def test_probe_atomics_count_exactly_inside_the_buffer(mib):
    torch = pytest.importorskip("torch")
    # guard band after the probed footprint: it must stay zero
    buf = torch.zeros((mib << 20) * 2, dtype=torch.uint8, device="cuda")
    st, issued = probe(buf.data_ptr(), mib << 20, 1, 1 << 22)
    assert st == N.OK, N.load().midsx_last_error()
    st0, issued0 = probe(buf.data_ptr(), mib << 20, 0, 1 << 22)
    assert st0 == N.OK
    torch.cuda.synchronize()
    words = buf.view(torch.int64).cpu().numpy()
    half = words.size // 2
    assert issued >= 1 << 22 and issued0 == issued
    assert int(words[:half].sum()) == issued
    assert not words[half:].any()
    # the hash spreads the requests: no sector takes more than a few times its share
    per_sector = words[:half].reshape(-1, 4)[:, 0]
    assert per_sector.max() <= max(16, 8 * issued // per_sector.size)
    assert np.count_nonzero(per_sector) >= min(per_sector.size, issued) // 2
