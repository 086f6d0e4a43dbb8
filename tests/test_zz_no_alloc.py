"""The allocation-free stage-A entry point (wb_assemble_li_noalloc).

Callers that may not allocate device memory — code running while another component captures a
CUDA graph, server plugins whose host owns the device pool, allocation-free real-time paths —
use this entry point; its scratch is a fixed device array inside the library. These tests call
it through the C ABI and hold its output to the handle-based wb_assemble_li on two calls in a
row (the shared scratch keeps the previous call's contents), and check that an oversized layer
is refused before any GPU work. This file is collected last on purpose.
"""
import numpy as np
import pytest

torch = pytest.importorskip('torch')

pytestmark = pytest.mark.gpu


def _setup():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300 import _lib, engine
    return _lib, _lib.load(), engine


def _raster(rng, L, ny, nx):
    eps = np.ones((L, ny, nx), complex)
    eps[rng.random((L, ny, nx)) < 0.4] = 12.25
    eps[rng.random((L, ny, nx)) < 0.1] = -20 + 1.5j
    return eps


def test_noalloc_assembly_matches_the_handle_entry_point_twice():
    _lib, lib, E = _setup()
    rng = np.random.default_rng(77)
    hu, hv = 4, 3
    N = (2 * hu + 1) * (2 * hv + 1)
    for call in range(2):
        ny, nx = (24, 20) if call == 0 else (17, 31)
        L = 3 if call == 0 else 2
        eps = torch.as_tensor(_raster(rng, L, ny, nx), device='cuda')
        want = E.assemble(eps, hu, hv)
        planes = torch.zeros((3, L, N, N), dtype=torch.complex128, device='cuda')
        status = torch.zeros(1, dtype=torch.int32, device='cuda')
        stream = torch.cuda.current_stream().cuda_stream
        rc = lib.wb_assemble_li_noalloc(eps.data_ptr(), L, ny, nx, hu, hv, planes[0].data_ptr(),
                                        planes[1].data_ptr(), planes[2].data_ptr(), status.data_ptr(), stream)
        assert rc == _lib.WB_OK, _lib.last_error()
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        for k in range(3):
            got = planes[k].transpose(-1, -2)
            ref = want.slot(k)
            scale = ref.abs().max().item()
            assert (got - ref).abs().max().item() <= 1e-12 * scale, (call, k)


def test_noalloc_refuses_a_layer_larger_than_its_scratch():
    """A 256x256 raster at orders (15, 15) is a valid request (N = 961) whose one-layer scratch,
    about 38 MiB, exceeds the fixed 32 MiB array: it is refused by the scratch check itself, before
    any GPU work, with a message that names the scratch."""
    _lib, lib, _ = _setup()
    limit = int(lib.wb_assemble_li_noalloc_limit())
    assert limit == 32 << 20
    eps = torch.ones((1, 256, 256), dtype=torch.complex128, device='cuda')
    out = torch.zeros(1, dtype=torch.complex128, device='cuda')
    rc = lib.wb_assemble_li_noalloc(eps.data_ptr(), 1, 256, 256, 15, 15, out.data_ptr(), out.data_ptr(),
                                    out.data_ptr(), None, torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.WB_E_INVALID
    assert 'scratch' in _lib.last_error()


def test_noalloc_accepts_the_largest_orders_that_fit():
    """The same raster at orders (14, 14) needs about 30 MiB of scratch and is assembled; its
    slots equal the handle-based entry point's."""
    _lib, lib, E = _setup()
    rng = np.random.default_rng(5)
    hu = hv = 14
    N = (2 * hu + 1) * (2 * hv + 1)
    eps = torch.as_tensor(_raster(rng, 1, 256, 256), device='cuda')
    want = E.assemble(eps, hu, hv)
    planes = torch.zeros((3, 1, N, N), dtype=torch.complex128, device='cuda')
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    rc = lib.wb_assemble_li_noalloc(eps.data_ptr(), 1, 256, 256, hu, hv, planes[0].data_ptr(), planes[1].data_ptr(),
                                    planes[2].data_ptr(), status.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.WB_OK, _lib.last_error()
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    for k in range(3):
        got = planes[k].transpose(-1, -2)
        ref = want.slot(k)
        assert (got - ref).abs().max().item() <= 1e-12 * ref.abs().max().item(), k
