"""qg_dot_noalloc: the inner-product entry point for callers that cannot allocate device
memory (for example a serving loop that has given all device memory to admitted jobs, or code
that must not risk the device-wide synchronisation cudaMalloc/cudaFree can cause).  It must
give qg_dot's results on two calls in a row, the second smaller than the first (the shared
scratch array keeps the first call's partial sums), and reject more vectors than its fixed
scratch holds.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_dot_noalloc_matches_qg_dot_on_two_calls():
    import torch
    from quanty_gb300 import build, qgpu
    build.build()
    L = qgpu.load()
    torch.cuda.set_device(0)
    ctx = ctypes.c_void_p()
    assert L.qg_init(0, ctypes.byref(ctx)) == 0
    stream = torch.cuda.Stream()
    assert L.qg_set_stream(ctx, ctypes.c_void_p(stream.cuda_stream)) == 0
    try:
        for n, nvec, seed in [(1_000_003, 3, 1), (77_777, 5, 2)]:
            rng = np.random.default_rng(seed)
            xh = rng.normal(size=(n, nvec)) + 1j * rng.normal(size=(n, nvec))
            yh = rng.normal(size=(n, nvec)) + 1j * rng.normal(size=(n, nvec))
            with torch.cuda.stream(stream):
                x = torch.from_numpy(xh).cuda()
                y = torch.from_numpy(yh).cuda()
                out = torch.zeros(nvec, dtype=torch.complex128, device="cuda")
            stream.synchronize()
            st = L.qg_dot_noalloc(n, nvec, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                  ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
            assert st == 0
            stream.synchronize()
            got = out.cpu().numpy()
            ref = np.zeros(2 * nvec)
            assert L.qg_dot(ctx, n, nvec, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                            ctypes.c_void_p(ref.ctypes.data)) == 0
            ref = ref[0::2] + 1j * ref[1::2]
            assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
            host = np.einsum("rk,rk->k", np.conj(xh), yh)
            assert np.max(np.abs(got - host)) <= 1e-10 * np.max(np.abs(host))
        # beyond the fixed scratch: a clear argument error, nothing launched
        big = torch.zeros((10, 65), dtype=torch.complex128, device="cuda")
        outb = torch.zeros(65, dtype=torch.complex128, device="cuda")
        assert L.qg_dot_noalloc(10, 65, ctypes.c_void_p(big.data_ptr()), ctypes.c_void_p(big.data_ptr()),
                                ctypes.c_void_p(outb.data_ptr()), ctypes.c_void_p(stream.cuda_stream)) == 4
    finally:
        L.qg_finalize(ctx)
