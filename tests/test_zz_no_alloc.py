"""snisr_render_rays_noalloc: the render entry point for callers that may not
allocate device memory while rendering (hosts that hand out all device
memory from their own pool, real-time frame loops that must not block on the
allocator).  Its scratch is a static device array; its results must equal the
allocating entry point's (snisr_render_rays, plain FP32 form) on the same
rays, call after call.  Collected last so that a stop-at-first-failure run has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

import oracle
import snisr
from snisr import _lib

pytestmark = pytest.mark.gpu

TOL = 1e-5  # same tolerance as the plain-form parity tests (bit-exact expected)


def test_noalloc_matches_allocating_entry_point(cuda):
    import torch
    s = snisr.SynthScene(snisr.CFG1)
    sc = snisr.Scene(s.desc)
    L = snisr.lib()
    stream = torch.cuda.current_stream().cuda_stream
    for call, pose in enumerate((0, 4)):  # two calls in a row (the scratch keeps the last call's contents)
        cam = s.camera(pose)
        d = oracle.camera_dirs(cam)
        n = 20000 + 3000 * call
        d = np.ascontiguousarray(d[:: d.shape[0] // n][:n])  # rays spread over the whole frame
        o = oracle.camera_origins(cam, n)
        od, dd = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
        ref = [torch.empty(n, 3, device=cuda), torch.empty(n, device=cuda), torch.empty(n, device=cuda)]
        out = [torch.full((n, 3), -7.0, device=cuda), torch.full((n,), -7.0, device=cuda),
               torch.full((n,), -7.0, device=cuda)]
        _lib.check(L.snisr_render_rays(sc.handle, od.data_ptr(), dd.data_ptr(), n, snisr.FORM_PLAIN_FP32,
                                       ref[0].data_ptr(), ref[1].data_ptr(), ref[2].data_ptr(), stream))
        _lib.check(L.snisr_render_rays_noalloc(sc.handle, od.data_ptr(), dd.data_ptr(), n, out[0].data_ptr(),
                                               out[1].data_ptr(), out[2].data_ptr(), stream))
        torch.cuda.synchronize()
        for a, b in zip(out, ref):
            assert float((a - b).abs().max()) <= TOL
        assert float(ref[2].max()) > 0.1  # the rays hit something
    # the property the entry point exists for: once set up, calls allocate
    # no device memory (the device's free bytes do not move over many calls)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(8):
        _lib.check(L.snisr_render_rays_noalloc(sc.handle, od.data_ptr(), dd.data_ptr(), n, out[0].data_ptr(),
                                               out[1].data_ptr(), out[2].data_ptr(), stream))
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    for a, b in zip(out, ref):
        assert float((a - b).abs().max()) <= TOL
    # sizes beyond the static scratch are rejected with a clear error
    st = L.snisr_render_rays_noalloc(sc.handle, od.data_ptr(), dd.data_ptr(), 32769, out[0].data_ptr(),
                                     out[1].data_ptr(), out[2].data_ptr(), stream)
    assert st == _lib.INVALID_ARG and b"32768" in L.snisr_last_error_string()
    sc.close()
