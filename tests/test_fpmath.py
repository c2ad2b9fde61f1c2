"""Accuracy of the pinned single-precision functions of include/sppm_fpmath.h (host evaluation,
the same code the kernels run) against double-precision numpy."""
import numpy as np

from oracle.binding import fpmath


def ulps(got, ref):
    ref32 = ref.astype(np.float32)
    spacing = np.spacing(np.abs(ref32)).astype(np.float64)
    return np.abs(got.astype(np.float64) - ref) / spacing


def test_sin_cos_within_2_ulp_on_the_shader_range():
    x = np.linspace(0.0, 6.283184, 400001, dtype=np.float32)
    for fn, ref in ((0, np.sin), (1, np.cos)):
        got = fpmath(fn, x)
        r = ref(x.astype(np.float64))
        big = np.abs(r) > 1e-3
        assert ulps(got[big], r[big]).max() <= 2.0
        assert np.abs(got - r).max() < 2e-7


def test_exp_within_2_ulp():
    x = np.linspace(-80.0, 80.0, 400001, dtype=np.float32)
    got = fpmath(3, x)
    r = np.exp(x.astype(np.float64))
    assert ulps(got, r).max() <= 2.0


def test_log2_exp2_pow_accuracy():
    rng = np.random.default_rng(1)
    x = rng.random(200000, dtype=np.float32) + np.float32(1e-6)
    l = fpmath(4, x)
    r = np.log2(x.astype(np.float64))
    ok = np.abs(r) > 1e-3
    assert ulps(l[ok], r[ok]).max() <= 4.0
    t = (rng.random(200000, dtype=np.float32) * 40 - 20).astype(np.float32)
    assert ulps(fpmath(5, t), np.exp2(t.astype(np.float64))).max() <= 2.0
    # pow(x, y) for the shader's uses: rnd^g (g < 1) and the sRGB exponent; error grows with
    # |y log2 x| (the exponent is rounded to single precision)
    y = (rng.random(200000, dtype=np.float32) * 3).astype(np.float32)
    p = fpmath(2, x, y)
    rp = np.power(x.astype(np.float64), y.astype(np.float64))
    tol = 2.0 + 1.5 * np.abs(y.astype(np.float64) * np.log2(x.astype(np.float64)))
    assert np.all(ulps(p, rp) <= tol)


def test_special_values():
    z = np.array([0.0, 1.0, np.inf, np.nan], np.float32)
    s = fpmath(0, z)
    assert s[0] == 0.0 and np.isnan(s[2]) and np.isnan(s[3])
    assert fpmath(2, np.array([0.0, 1.0, 2.0], np.float32), np.array([2.0, 5.0, 0.0], np.float32)).tolist() == [0.0, 1.0, 1.0]
    assert fpmath(3, np.array([-200.0, 200.0], np.float32)).tolist() == [0.0, np.inf]
