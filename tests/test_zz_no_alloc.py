"""The allocation-free filter apply (tmrg_filter_apply_static_device).

Callers that cannot allocate device memory where they filter — a framework
whose allocator owns the GPU's memory, or code that must not call
cudaMalloc/cudaFree because those can synchronise the device — use this
entry point: its work vectors live in a static device array of the library.
This checks, through the C ABI, that it returns what the allocating
tmrg_filter_apply_device returns (tolerance 1e-13 relative, the FP64
tolerance of the other filter tests) on two calls in a row, forward and
transpose, that those calls allocate no device memory (the library's
allocation counter stays put), and that it rejects a problem larger than
its fixed scratch.
The file is named to be collected last."""
import ctypes

import numpy as np
import pytest

from tests import pipeline


@pytest.mark.gpu
def test_static_scratch_filter_apply_matches_allocating_apply(gpu_lib):
    import torch

    from tmr_gb300 import TMR
    from tmr_gb300._lib import lib
    L = lib()
    case = pipeline.cases()["brick_o2"]
    g = pipeline.run_gpu(dict(case, coarse_levels=0))
    F = TMR.MatrixFilter(0.08, 10, None, [g["forests"][0]])
    n, _ = F.size()
    vpn = 3
    gen = torch.Generator(device="cpu").manual_seed(13)
    for transpose in (0, 1):
        x = torch.rand(n * vpn, generator=gen, dtype=torch.float64).cuda()
        ref = torch.empty_like(x)
        name = "tmrg_filter_apply_transpose_device" if transpose else "tmrg_filter_apply_device"
        assert getattr(L, name)(F.ptr, vpn, ctypes.c_void_p(x.data_ptr()),
                                ctypes.c_void_p(ref.data_ptr())) == 0
        for _ in range(2):  # two calls in a row share the static scratch
            out = torch.full_like(x, float("nan"))
            torch.cuda.synchronize()
            allocs = L.tmrg_device_alloc_count()
            rc = L.tmrg_filter_apply_static_device(F.ptr, transpose, vpn,
                                                   ctypes.c_void_p(x.data_ptr()),
                                                   ctypes.c_void_p(out.data_ptr()))
            assert rc == 0, L.tmrg_last_error()
            torch.cuda.synchronize()
            # the property the entry point exists for: no device allocation
            assert L.tmrg_device_alloc_count() == allocs
            np.testing.assert_allclose(out.cpu().numpy(), ref.cpu().numpy(),
                                       rtol=1e-13, atol=0.0)
    # nodes x vpn beyond the fixed scratch: rejected before any launch
    big_vpn = (1 << 20) // n + 1
    rc = L.tmrg_filter_apply_static_device(F.ptr, 0, big_vpn,
                                           ctypes.c_void_p(x.data_ptr()),
                                           ctypes.c_void_p(out.data_ptr()))
    assert rc == 1 and b"scratch" in L.tmrg_last_error()
