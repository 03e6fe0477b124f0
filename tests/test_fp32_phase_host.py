"""The precision form's phase arithmetic, emulated on the host in float32
(no GPU): sincos_2pi (quadrant reduction + Maclaurin series) and
sincos_turns (float-float phase in turns, integer turns removed exactly),
as written in csrc/phk_device.cuh; the paired-pipe forms run the same
operations lane by lane.  fmaf is emulated as one rounding of the exact
float64 product-sum (exact for float32 products), which matches the device
up to rare double-rounding ties.

Checked: sin/cos(2 pi f) within 2 float32 ulps of the float64 value
(measured 0.57 ulp at most over 4e5 arguments); no sign bias of
sin^2 + cos^2 - 1 (measured mean -0.005 ulp, spread 0.29 ulp; a bias would
grow betatron amplitudes secularly); the float-float phase of a tune near 20 reproduces
sin/cos(2 pi (Q + d)) at the float32 rounding of the result, where a
plain float32 phase is off by ~1e-6."""
import numpy as np

f32 = np.float32


def fmaf(a, b, c):
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64)
            + np.asarray(c, np.float64)).astype(np.float32)


def sincos_2pi(f):
    f = np.asarray(f, np.float32)
    q = np.rint(f32(4) * f).astype(np.float32)
    r = fmaf(f32(-0.25), q, f)
    th = fmaf(r, f32(6.28318548202514648438), r * f32(-1.7484556e-7))
    t2 = th * th
    ps = fmaf(t2, f32(-2.5052108385e-8), f32(2.7557319224e-6))
    ps = fmaf(t2, ps, f32(-1.9841269841e-4))
    ps = fmaf(t2, ps, f32(8.3333333333e-3))
    ps = fmaf(t2, ps, f32(-1.6666666667e-1))
    sn = fmaf(th * t2, ps, th)
    pc = fmaf(t2, f32(-2.7557319224e-7), f32(2.4801587302e-5))
    pc = fmaf(t2, pc, f32(-1.3888888889e-3))
    pc = fmaf(t2, pc, f32(4.1666666667e-2))
    pc = fmaf(t2, pc, f32(-0.5))
    cs = fmaf(t2, pc, f32(1))
    k = q.astype(np.int64) & 3
    a = np.where(k & 1, cs, sn)
    b = np.where(k & 1, sn, cs)
    s = np.where(k & 2, -a, a)
    c = np.where((k + 1) & 2, -b, b)
    return s.astype(np.float32), c.astype(np.float32)


def sincos_turns(hi, lo, d):
    hi, lo, d = (np.asarray(v, np.float32) for v in (hi, lo, d))
    t = hi + d
    bp = t - hi
    err = (hi - (t - bp)) + (d - bp)
    err = err + lo
    r = t - np.rint(t).astype(np.float32)
    f = r + err
    g = (r - f) + err
    sp, cp = sincos_2pi(f)
    dl = f32(6.28318530717958647692) * g
    return fmaf(dl, cp, sp), fmaf(-dl, sp, cp)


def test_sincos_2pi_accuracy_and_no_bias():
    rng = np.random.RandomState(1)
    f = rng.uniform(-0.5, 0.5, 400000).astype(np.float32)
    s, c = sincos_2pi(f)
    th = 2 * np.pi * f.astype(np.float64)
    ulp = np.finfo(np.float32).eps
    assert np.max(np.abs(s - np.sin(th))) <= 2 * ulp
    assert np.max(np.abs(c - np.cos(th))) <= 2 * ulp
    n2 = s.astype(np.float64)**2 + c.astype(np.float64)**2 - 1
    # the rounding of s and c alone gives an unbiased spread of ~ulp
    assert abs(np.mean(n2)) < 0.02 * ulp, np.mean(n2)
    # quadrant boundaries and exact quarter turns
    q = np.array([-0.5, -0.375, -0.25, -0.125, 0., 0.125, 0.25, 0.375, 0.5],
                 np.float32)
    s, c = sincos_2pi(q)
    np.testing.assert_allclose(s, np.sin(2 * np.pi * q.astype(np.float64)),
                               atol=2 * ulp)
    np.testing.assert_allclose(c, np.cos(2 * np.pi * q.astype(np.float64)),
                               atol=2 * ulp)


def test_float_float_phase_keeps_the_tune():
    """The base tune Q (frac part, float-float) plus a float detuning d: the
    result follows sin/cos(2 pi (Q + d)) to the float32 rounding, i.e. the
    tune carries no float32 rounding error turn after turn."""
    rng = np.random.RandomState(2)
    Q = 20.13
    frac = Q - np.floor(Q)
    hi = np.float32(frac)
    lo = np.float32(frac - np.float64(hi))
    d = rng.normal(0, 5e-3, 200000).astype(np.float32)
    s, c = sincos_turns(np.full_like(d, hi), np.full_like(d, lo), d)
    ph = 2 * np.pi * (frac + d.astype(np.float64))
    ulp = np.finfo(np.float32).eps
    es = np.abs(s - np.sin(ph))
    ec = np.abs(c - np.cos(ph))
    assert max(es.max(), ec.max()) <= 2 * ulp
    # systematic phase error (mean over particles) far below one ulp
    dphi = np.mean((s - np.sin(ph)) * np.cos(ph) - (c - np.cos(ph)) * np.sin(ph))
    assert abs(dphi) < 0.05 * ulp, dphi
    # a plain float32 phase of the full tune loses ~1e-6 of a radian
    s32 = np.sin((np.float32(2 * np.pi) * (np.float32(Q) + d)).astype(np.float64))
    assert np.max(np.abs(s32 - np.sin(2 * np.pi * (Q + d.astype(np.float64))))) > 1e-6
