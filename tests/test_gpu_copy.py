"""GPU test of clmgb_copy_segments: device to page-locked host, host to device and
device to device segments in one call, empty and single-word segments, and the
argument checks (misaligned, odd sizes, pageable host memory, too many segments)."""
import ctypes as C

import numpy as np
import pytest

from clmgb import abi, api, hoststep

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _call(h, dst, src, nbytes, n=None):
    n = len(dst) if n is None else n
    d = (C.c_void_p * max(1, len(dst)))(*dst)
    s = (C.c_void_p * max(1, len(src)))(*src)
    b = (C.c_int64 * max(1, len(nbytes)))(*nbytes)
    return h.lib.clmgb_copy_segments(d, s, b, n, C.c_void_p(torch.cuda.current_stream().cuda_stream))


def test_copy_segments_moves_every_segment():
    h = api.Handle(abi.Varpar(12, 25, 20, 5, 25, 0))
    try:
        g = torch.Generator(device="cuda").manual_seed(3)
        sizes = [0, 1, 7, 1000, 123457, 3 * 152 * 256 * 4 + 5]
        dev = [torch.rand(n, dtype=torch.float64, device="cuda", generator=g) for n in sizes]
        host = [torch.empty(n, dtype=torch.float64).pin_memory() for n in sizes]
        hoststep.copy_segments(h, list(zip(host, dev)), torch.cuda.current_stream())
        back = [torch.full((n,), -1.0, dtype=torch.float64, device="cuda") for n in sizes]
        dd = [torch.empty(n, dtype=torch.float64, device="cuda") for n in sizes]
        hoststep.copy_segments(h, list(zip(back, host)) + list(zip(dd, dev)), torch.cuda.current_stream())
        torch.cuda.synchronize()
        for a, b, c, e in zip(dev, host, back, dd):
            assert torch.equal(a.cpu(), b) and torch.equal(a, c) and torch.equal(a, e)
        ints = torch.arange(10001, dtype=torch.int64, device="cuda")
        ih = torch.zeros(10001, dtype=torch.int64).pin_memory()
        hoststep.copy_segments(h, [(ih, ints)], torch.cuda.current_stream())
        torch.cuda.synchronize()
        assert np.array_equal(ih.numpy(), np.arange(10001))
    finally:
        h.close()


def test_copy_segments_checks_its_arguments():
    h = api.Handle(abi.Varpar(12, 25, 20, 5, 25, 0))
    try:
        a = torch.zeros(64, dtype=torch.float64, device="cuda")
        b = torch.zeros(64, dtype=torch.float64, device="cuda")
        pageable = np.zeros(64)
        assert _call(h, [a.data_ptr()], [b.data_ptr()], [512]) == abi.CLMGB_OK
        assert _call(h, [a.data_ptr() + 4], [b.data_ptr()], [8]) == abi.CLMGB_ERR_DIMS
        assert _call(h, [a.data_ptr()], [b.data_ptr()], [12]) == abi.CLMGB_ERR_DIMS
        assert _call(h, [a.data_ptr()], [b.data_ptr()], [-8]) == abi.CLMGB_ERR_DIMS
        assert _call(h, [pageable.ctypes.data], [b.data_ptr()], [64]) == abi.CLMGB_ERR_DIMS
        assert _call(h, [a.data_ptr()], [0], [8]) == abi.CLMGB_ERR_NULL_ARG
        assert _call(h, [a.data_ptr()], [b.data_ptr()], [8], n=abi.MAX_COPY_SEGMENTS + 1) == abi.CLMGB_ERR_DIMS
        assert _call(h, [], [], [], n=0) == abi.CLMGB_OK
        torch.cuda.synchronize()
        assert h.device_status() == 0
    finally:
        h.close()
