"""The bulk-copy primitives in isolation (sph_selftest_staging): a bulk
asynchronous copy that completes on an mbarrier, and a bounded wait on bytes
that never arrive, which must give up and report instead of hanging."""
import ctypes as C

import pytest
import torch

pytestmark = pytest.mark.gpu


def test_bulk_copy_lands_and_bounded_wait_gives_up():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sph import _lib, build
    build.build()
    lib = _lib.load()
    src = torch.arange(16, dtype=torch.float32, device="cuda") * 0.5 + 1.0
    res = torch.zeros(2, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.sph_selftest_staging(src.data_ptr(), res.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    assert res.tolist() == [1, 2]
    # a misaligned source is rejected on the host
    assert lib.sph_selftest_staging(src.data_ptr() + 4, res.data_ptr(), stream) == 1
