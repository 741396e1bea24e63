"""The FP32 far field's wave-front margin, checked against an FP32 emulation on CPU.

The far kernel computes tau = T - r/c in FP32 from element-relative offsets (the
node's offset from FP32 coordinate pairs, the Gauss point's from the FP32 table),
r = r2 * rsqrtf(r2) and FP32 T = k dt and 1/c.  Within kTauMargin (T + dt + r/c_p)
of a threshold (kTauMargin = 64 / 2^24) it takes the regime decisions from FP64
(assemble.cu: gauss_point_f32, front_taus); that is safe when the FP32 tau is never
off by more than the margin.  This emulates the kernel's arithmetic in float32
(rsqrtf as the float32 reciprocal square root off by up to 2 ulp) over random
geometries and levels and checks that the error stays within a quarter of the
margin (observed: at most a tenth).
"""
import numpy as np

EPS32 = 2.0 ** -24
MARGIN = 64 * EPS32


def pair32(x):
    hi = x.astype(np.float32)
    return hi, (x - hi.astype(np.float64)).astype(np.float32)


def test_fp32_tau_error_is_well_inside_the_margin():
    rng = np.random.default_rng(0)
    n = 200000
    cp, cs, dt = np.sqrt(3.0), 1.0, 0.6 * (np.pi / 32) / np.sqrt(3.0)
    # node and element first node on a unit sphere, the Gauss point near the element
    def on_sphere(k):
        v = rng.standard_normal((k, 3))
        return v / np.linalg.norm(v, axis=1, keepdims=True)
    xc = on_sphere(n)
    xe = on_sphere(n)
    xq = xe + 0.1 * rng.standard_normal((n, 3))
    k = rng.integers(0, 92, n)

    # FP64 reference, as the FP64 quadrature computes it
    r64 = np.linalg.norm(xq - xc, axis=1)
    T64 = k * dt
    tp64 = T64 - r64 / cp

    # FP32 emulation of the far kernel
    ch, cl = pair32(xc)
    eh, el = pair32(xe)
    xc_rel = (ch - eh) + (cl - el)                                 # float32
    xq_rel = (xq - xe).astype(np.float32)                           # the FP32 table
    d = xq_rel - xc_rel
    r2 = np.sum(d * d, axis=1, dtype=np.float32)
    inv_r = (1.0 / np.sqrt(r2.astype(np.float64))).astype(np.float32)
    ulp = np.spacing(inv_r)
    inv_r = inv_r + rng.integers(-2, 3, n).astype(np.float32) * ulp  # rsqrtf: <= 2 ulp
    r = r2 * inv_r
    dt32, icp = np.float32(dt), np.float32(1.0 / cp)
    TI = k.astype(np.float32) * dt32
    tp32 = TI - r * icp

    err = np.abs(tp32.astype(np.float64) - tp64)
    margin = MARGIN * (TI.astype(np.float64) + dt + r64 / cp)
    assert np.all(err <= margin / 4), (err / margin).max()
