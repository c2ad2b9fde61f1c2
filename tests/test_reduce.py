"""ReduceTexture (glslppm.cpp:170-209): the oracle's restatement equals the reference's min.fs /
max.fs / sum.fs driven through the ping-pong scheme (reference marker), and the CUDA stage entry
point sppm_reduce_texture equals the oracle bit for bit (gpu marker)."""
import ctypes as C

import numpy as np
import pytest

from oracle.binding import reduce_texture as oracle_reduce


def textures():
    rng = np.random.default_rng(11)
    for R in (2, 4, 8, 64, 256):
        t = (rng.standard_normal((R * R, 4)) * 100).astype(np.float32)
        yield R, t
    # the reference's use: emitted-photon flags (0/1) and hit positions with zeros for misses
    R = 128
    flags = (rng.random((R * R, 4)) < 0.3).astype(np.float32)
    yield R, flags


@pytest.mark.reference
def test_oracle_reduce_equals_reference_shaders():
    from oracle.build import REF_DIR, build_ref
    build_ref()
    lib = C.CDLL(str(REF_DIR / "libref_shaders.so"))
    lib.ref_gl_reduce.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    for R, t in textures():
        for op in (0, 1, 2):
            ref = np.zeros(4, np.float32)
            lib.ref_gl_reduce(t.ctypes.data, R, op, ref.ctypes.data)
            assert np.array_equal(oracle_reduce(t, R, op).view(np.uint32), ref.view(np.uint32)), (R, op)


def test_oracle_reduce_semantics():
    rng = np.random.default_rng(2)
    t = rng.random((64 * 64, 4)).astype(np.float32)
    assert np.array_equal(oracle_reduce(t, 64, 0), t.min(axis=0))
    assert np.array_equal(oracle_reduce(t, 64, 1), t.max(axis=0))
    assert np.allclose(oracle_reduce(t, 64, 2), t.astype(np.float64).sum(axis=0), rtol=1e-5)
    with pytest.raises(ValueError):
        oracle_reduce(t, 63, 0)


@pytest.mark.gpu
def test_cuda_reduce_texture_bit_exact():
    torch = pytest.importorskip("torch")
    import glslppm_gb300 as g
    for R, t in textures():
        d = torch.from_numpy(t).cuda()
        for op in (0, 1, 2):
            got = g.renderer.reduce_texture(d.data_ptr(), R, op, torch.cuda.current_stream().cuda_stream)
            assert np.array_equal(got.view(np.uint32), oracle_reduce(t, R, op).view(np.uint32)), (R, op)


@pytest.mark.gpu
def test_cuda_reduce_texture_rejects_bad_sizes():
    torch = pytest.importorskip("torch")
    import glslppm_gb300 as g
    from glslppm_gb300 import native as N
    d = torch.zeros((48 * 48, 4), device="cuda")
    with pytest.raises(N.SppmError) as e:
        g.renderer.reduce_texture(d.data_ptr(), 48, 0)
    assert e.value.status == N.ERR_ARG
