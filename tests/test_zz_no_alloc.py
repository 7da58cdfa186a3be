"""rtx_image_gaussian_blur_noalloc: the Gaussian blur for callers that cannot
allocate device memory when they call in (a plugin whose host application owns
the device-memory budget, a real-time loop that must not synchronise the
device).  It keeps its intermediate image in a fixed device array instead of
allocating one.

Called through the C ABI several times in a row on device buffers the test
owns -- out of place, in place with the largest kernel, and captured into a
CUDA graph and replayed; each result must equal, bit for bit, what
rtx_image_gaussian_blur returns for the same image (the tolerance of every
compositor test here).  Collected last so a failing run has already run every
other test; it also passes alone.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_blur_matches_allocating_entry_point():
    import torch

    import rendertoy_gb300 as rt
    from rendertoy_gb300 import build
    build.build()
    L = rt.lib()
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream().cuda_stream
    msg = C.create_string_buffer(256)
    ctx = rt.Context(0)
    try:
        rng = np.random.RandomState(12)
        cases = [(300, 200, 49, 8.0), (1024, 1024, 7, 1.5)]
        for W, H, size, sigma in cases:  # two calls in a row, different sizes
            img = rng.exponential(0.7, (H, W, 3)).astype(np.float32)
            d_in = torch.from_numpy(img).cuda()
            d_out = torch.full_like(d_in, float("nan"))
            r = L.rtx_image_gaussian_blur_noalloc(C.c_void_p(d_in.data_ptr()),
                                                  C.c_void_p(d_out.data_ptr()), W, H, size,
                                                  sigma, C.c_void_p(stream), msg, len(msg))
            assert r == 0, msg.value
            torch.cuda.synchronize()
            want = ctx.gaussian_blur(img, size, sigma)
            got = d_out.cpu().numpy()
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (W, H, size)
        # in place (d_in == d_out) with the largest kernel: its column pass
        # needs more than the default 48 KB of shared memory
        img = rng.exponential(0.7, (96, 160, 3)).astype(np.float32)
        d_io = torch.from_numpy(img).cuda()
        r = L.rtx_image_gaussian_blur_noalloc(C.c_void_p(d_io.data_ptr()), C.c_void_p(d_io.data_ptr()),
                                              160, 96, 255, 40.0, C.c_void_p(stream), msg, len(msg))
        assert r == 0, msg.value
        torch.cuda.synchronize()
        want = ctx.gaussian_blur(img, 255, 40.0)
        assert np.array_equal(d_io.cpu().numpy().view(np.uint32), want.view(np.uint32))
        # sizes beyond the fixed scratch are refused, with a message
        big = torch.zeros((2049, 1024, 3), device="cuda")
        r = L.rtx_image_gaussian_blur_noalloc(C.c_void_p(big.data_ptr()), C.c_void_p(big.data_ptr()),
                                              1024, 2049, 7, 1.5, C.c_void_p(stream), msg, len(msg))
        assert r == 1 and b"scratch" in msg.value
        r = L.rtx_image_gaussian_blur_noalloc(C.c_void_p(big.data_ptr()), C.c_void_p(big.data_ptr()),
                                              64, 64, 256, 1.5, C.c_void_p(stream), msg, len(msg))
        assert r == 1
        # within the pixel limit but taller than a grid's rows: refused too
        tall = torch.zeros((70000, 16, 3), device="cuda")
        r = L.rtx_image_gaussian_blur_noalloc(C.c_void_p(tall.data_ptr()), C.c_void_p(tall.data_ptr()),
                                              16, 70000, 7, 1.5, C.c_void_p(stream), msg, len(msg))
        assert r == 1 and b"65535" in msg.value
        # captured into a CUDA graph on a stream of its own (after one call on
        # that stream outside the capture) and replayed: the same bits
        img = rng.exponential(0.7, (256, 384, 3)).astype(np.float32)
        d_in = torch.from_numpy(img).cuda()
        d_out = torch.full_like(d_in, float("nan"))
        side = torch.cuda.Stream()

        def call():
            return L.rtx_image_gaussian_blur_noalloc(C.c_void_p(d_in.data_ptr()), C.c_void_p(d_out.data_ptr()),
                                                     384, 256, 49, 8.0, C.c_void_p(side.cuda_stream), msg,
                                                     len(msg))
        torch.cuda.synchronize()
        with torch.cuda.stream(side):
            assert call() == 0, msg.value
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=side):
            r = call()
        assert r == 0, msg.value
        d_out.fill_(float("nan"))
        graph.replay()
        torch.cuda.synchronize()
        want = ctx.gaussian_blur(img, 49, 8.0)
        assert np.array_equal(d_out.cpu().numpy().view(np.uint32), want.view(np.uint32))
    finally:
        ctx.close()
