"""sppm_reduce_texture_noalloc -- ReduceTexture for callers that must not allocate device memory
(for example an engine that reserved the GPU's memory for its own allocator, or a render loop that
forbids allocation once it runs).  It works in a fixed scratch array inside the library instead of
allocating one per call.

Called through the C ABI, it must return exactly what the allocating entry point
sppm_reduce_texture returns, on two calls in a row (the scratch keeps the previous call's
contents), must not change the device's free memory, and must refuse a texture larger than its
scratch.  This file is collected last so that a run stopping at the first failure has run every
other test first.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def call(fn, ptr, resolution, op, stream):
    out = (C.c_float * 4)()
    st = fn(ptr, resolution, op, out, stream)
    return st, np.array(list(out), dtype=np.float32)


@pytest.mark.parametrize("op", [0, 1, 2], ids=["min", "max", "sum"])
def test_no_alloc_reduce_matches_the_allocating_entry_point_twice(op):
    torch = pytest.importorskip("torch")
    from glslppm_gb300 import native as N
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(3 + op)
    # two calls in a row for each size: the second finds the first one's contents in the scratch;
    # resolution 2 runs a single level, 1024 is the largest the scratch holds
    resolutions = [1024, 1024, 256, 2, 2, 32]
    textures = [torch.from_numpy((rng.standard_normal((r * r, 4)) * 50).astype(np.float32)).cuda()
                for r in resolutions]
    expected = []
    for r, t in zip(resolutions, textures):
        st, ref = call(N.lib.sppm_reduce_texture, t.data_ptr(), r, op, stream)
        assert st == N.OK, N.last_error()
        expected.append(ref)
    # the first call on this device performs the one-time set-up (symbol address lookup)
    st, _ = call(N.lib.sppm_reduce_texture_noalloc, textures[2].data_ptr(), resolutions[2], (op + 1) % 3, stream)
    assert st == N.OK, N.last_error()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for r, t, ref in zip(resolutions, textures, expected):
        st, got = call(N.lib.sppm_reduce_texture_noalloc, t.data_ptr(), r, op, stream)
        assert st == N.OK, N.last_error()
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (r, op, got, ref)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before


def test_no_alloc_reduce_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from glslppm_gb300 import native as N
    t = torch.zeros((2048 * 2048, 4), device="cuda")
    st, _ = call(N.lib.sppm_reduce_texture_noalloc, t.data_ptr(), 2048, 0, torch.cuda.current_stream().cuda_stream)
    assert st == N.ERR_ARG
    assert "exceeds the maximum" in N.last_error()
