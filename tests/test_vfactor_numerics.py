"""Numerics of the FP32 vertical-diffusion factorisation (k32_vfactors), restated in numpy FP32:
the Thomas pivots m(k) = b(k) - a(k) c(k-1) / m(k-1) of the implicit solve
(src/oce_ale_tracer.F90:1406-1414), with a, c <= 0 and b = |a| + |c| + h, formed from their excess
d = m - |c| (d(k) = h(k) + |a(k)| d(k-1) / (d(k-1) + |c(k-1)|)) as the kernel does: by a scan of
the non-negative 2x2 linear-fractional maps of d over 32-level chunks, rescaled by powers of two.
Against the exact pivots of the same FP32 coefficients, the excess form keeps a few ulps on
columns with thin bottom cells under strong diffusion, where the textbook FP32 recurrence loses
most of its bits."""
import numpy as np

F = np.float32


def _mul(x, y):
    return np.array([[x[0, 0] * y[0, 0] + x[0, 1] * y[1, 0], x[0, 0] * y[0, 1] + x[0, 1] * y[1, 1]],
                     [x[1, 0] * y[0, 0] + x[1, 1] * y[1, 0], x[1, 0] * y[0, 1] + x[1, 1] * y[1, 1]]], dtype=F)


def _pow2_inv(x):
    return F(2.0) ** F(-(np.frexp(x)[1] - 1))


def pivots_scan(a, c, h):
    """The kernel's evaluation: per chunk of 32 levels an inclusive scan of the level maps
    (later level on the left), applied to the vector carried from the chunk above."""
    L = len(h)
    m = np.zeros(L, F)
    cx, cy = F(1), F(1)
    for k0 in range(0, L, 32):
        ks = list(range(k0, min(L, k0 + 32)))
        S = []
        for k in ks:
            S.append(np.array([[0, h[k]], [0, 1]], F) if k == 0 else
                     np.array([[h[k] - a[k], h[k] * -c[k - 1]], [1, -c[k - 1]]], F))
        S += [np.eye(2, dtype=F)] * (32 - len(ks))
        off = 1
        while off < 32:
            S = [(_mul(S[l], S[l - off]) * _pow2_inv(np.max(_mul(S[l], S[l - off])))).astype(F) if l >= off
                 else S[l] for l in range(32)]
            off *= 2
        for j, k in enumerate(ks):
            v0 = F(S[j][0, 0] * cx + S[j][0, 1] * cy)
            v1 = F(S[j][1, 0] * cx + S[j][1, 1] * cy)
            m[k] = F(v0 / v1) - c[k]
        w0 = F(S[31][0, 0] * cx + S[31][0, 1] * cy)
        w1 = F(S[31][1, 0] * cx + S[31][1, 1] * cy)
        sc = _pow2_inv(max(w0, w1))
        cx, cy = F(w0 * sc), F(w1 * sc)
    return m


def pivots_textbook32(a, c, h):
    m = np.zeros(len(h), F)
    for k in range(len(h)):
        b = F(F(-a[k] - c[k]) + h[k])
        m[k] = b if k == 0 else F(b - F(a[k] * F(c[k - 1] / m[k - 1])))
    return m


def pivots_exact(a, c, h):
    a, c, h = (np.asarray(x, np.float64) for x in (a, c, h))
    m = np.zeros(len(h))
    for k in range(len(h)):
        b = -a[k] - c[k] + h[k]
        m[k] = b if k == 0 else b - a[k] * c[k - 1] / m[k - 1]
    return m


def _column(rng, L):
    h = rng.uniform(1, 50, L)
    h[-int(rng.integers(1, min(4, L) + 1)):] *= 10.0 ** rng.uniform(-5, -1)  # thin bottom cells
    kv = 10.0 ** rng.uniform(-5, 0, L)
    a = -kv * 600.0 / rng.uniform(1, 50, L)
    a[0] = 0.0
    c = np.r_[a[1:], 0.0] * rng.uniform(0.5, 2.0, L)
    c[-1] = 0.0
    return a.astype(F), c.astype(F), h.astype(F)


def test_excess_form_scan_keeps_the_pivots_to_a_few_ulps():
    rng = np.random.default_rng(7)
    worst_scan, worst_text = 0.0, 0.0
    for _ in range(40):
        a, c, h = _column(rng, int(rng.integers(2, 100)))
        m = pivots_exact(a, c, h)
        worst_scan = max(worst_scan, float(np.max(np.abs(pivots_scan(a, c, h) - m) / m)))
        worst_text = max(worst_text, float(np.max(np.abs(pivots_textbook32(a, c, h) - m) / m)))
    assert worst_scan < 1e-6, worst_scan
    # the cancellation the excess form avoids
    assert worst_text > 1e-4, worst_text


def test_single_layer_and_uniform_columns():
    # one layer: m = h exactly; a column without diffusion: m = h to the rounding of the scan's
    # products and quotient (a couple of ulps)
    a, c, h = np.zeros(1, F), np.zeros(1, F), np.full(1, 7.0, F)
    assert pivots_scan(a, c, h)[0] == F(7.0)
    L = 70
    z = np.zeros(L, F)
    h = np.full(L, 3.0, F)
    assert np.max(np.abs(pivots_scan(z, z, h) - h) / h) <= 2.5e-7
