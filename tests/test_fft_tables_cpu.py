"""The FFT pass tables that chl_create stages (chl_fft_pass_table, built on
the host) against numpy.fft, without a GPU.

The device transform (chl_fft.cu: stockham_pass) takes each twiddle in
tangent form: w = sigma (1 + i m) with sigma = C and m = S/C where |C| >=
|S|, else w = sigma (m + i) with sigma = S and m = C/S, and folds the
sigmas into the butterflies' FMAs; the inverse transform flips signs of the
same table.  This test restates those butterflies in NumPy, reading every
multiplier, scale and form bit from the library's table, and checks both
directions of every length 2^a 3^b up to 256 against numpy.fft
(tolerance 1e-14 of the largest output).  It also checks the properties
the forms exist for: every multiplier within [-1, 1], every scale at least
1/sqrt(2) in magnitude.
"""
import numpy as np
import pytest

TWF = 7
LENGTHS = sorted({2 ** a * 3 ** b for a in range(9) for b in range(6) if 2 <= 2 ** a * 3 ** b <= 256})


def _radix(rem):
    return 4 if rem % 4 == 0 else (3 if rem % 3 == 0 else 2)


def _flip(x, f):
    return np.where(f, -x, x)


def _tw(v, m, sform):
    """v w / sigma: (a - b m) + i (b + a m) in the C form, (a m - b) + i (b m + a) in the S form."""
    a, b = v.real, v.imag
    re = np.where(sform, a * m - b, a - b * m)
    im = np.where(sform, b * m + a, b + a * m)
    return re + 1j * im


def _dft_small(v, R, inv):
    s = 1.0 if inv else -1.0
    w = np.exp(s * 2j * np.pi * np.outer(np.arange(R), np.arange(R)) / R)
    return [sum(w[k, q] * v[q] for q in range(R)) for k in range(R)]


def stockham(x, tab, inv):
    """The device's passes over the library's table (one transform of length len(x))."""
    N = len(x)
    src = np.asarray(x, complex)
    Ns, rem, off = 1, N, 0
    iv = 1 if inv else 0
    while rem > 1:
        R = _radix(rem)
        nb = N // R
        j = np.arange(nb)
        jm = j % Ns
        v = [src[j + r * nb] for r in range(R)]
        if Ns == 1:
            out = _dft_small(v, R, inv)
        else:
            t = tab[off:off + TWF * Ns].reshape(TWF, Ns)[:, jm]
            fb = t[6].view(np.int64)
            f1, f2, f3 = (fb >> 1) & 1, (fb >> 2) & 1, (fb >> 3) & 1
            s1 = _flip(t[3], iv & f1)
            y1 = _tw(v[1], _flip(t[0], iv), f1)
            if R == 2:
                out = [v[0] + s1 * y1, v[0] - s1 * y1]
            elif R == 4:
                y2 = _tw(v[2], _flip(t[1], iv), f2)
                y3 = _tw(v[3], _flip(t[2], iv), f3)
                s2 = _flip(t[4], iv & f2)
                rho = _flip(t[5], iv & (f1 ^ f3))
                a, b = v[0] + s2 * y2, v[0] - s2 * y2
                c, e = y1 + rho * y3, y1 - rho * y3
                si = _flip(s1, iv)
                out = [a + s1 * c, (b.real + si * e.imag) + 1j * (b.imag - si * e.real), a - s1 * c,
                       (b.real - si * e.imag) + 1j * (b.imag + si * e.real)]
            else:
                y2 = _tw(v[2], _flip(t[1], iv), f2)
                h1 = _flip(t[4], iv & f1)
                rho = _flip(t[5], iv & (f1 ^ f2))
                k1 = _flip(t[2], iv & (f1 ^ 1))
                sp, dp = y1 + rho * y2, y1 - rho * y2
                tt = v[0] - h1 * sp
                out = [v[0] + s1 * sp, (tt.real + k1 * dp.imag) + 1j * (tt.imag - k1 * dp.real),
                       (tt.real - k1 * dp.imag) + 1j * (tt.imag + k1 * dp.real)]
            off += TWF * Ns
        dst = np.empty(N, complex)
        idx = (j // Ns) * Ns * R + jm
        for r in range(R):
            dst[idx + r * Ns] = out[r]
        src = dst
        Ns *= R
        rem //= R
    assert off == len(tab)
    return src


@pytest.mark.parametrize("N", LENGTHS)
def test_pass_table_transforms_match_numpy(N):
    from channel_rl_gb300.host import fft_pass_table
    tab = fft_pass_table(N)
    rng = np.random.default_rng(N)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    for inv in (False, True):
        got = stockham(x, tab, inv)
        want = np.fft.ifft(x) * N if inv else np.fft.fft(x)
        assert np.abs(got - want).max() <= 1e-14 * np.abs(want).max(), (N, inv)


@pytest.mark.parametrize("N", [128, 192, 256, 162])
def test_pass_table_multipliers_and_scales(N):
    """|m| <= 1 and |sigma| >= 1/sqrt(2) for every twiddle of every pass."""
    from channel_rl_gb300.host import fft_pass_table
    tab = fft_pass_table(N)
    Ns, rem, off = 1, N, 0
    while rem > 1:
        R = _radix(rem)
        if Ns > 1:
            t = tab[off:off + TWF * Ns].reshape(TWF, Ns)
            ms = [t[0], t[1]] + ([t[2]] if R == 4 else [])
            assert all(np.all(np.abs(m) <= 1.0) for m in ms)
            assert np.all(np.abs(t[3]) >= 2 ** -0.5 - 1e-15)
            if R == 4:
                assert np.all(np.abs(t[4]) >= 2 ** -0.5 - 1e-15)
            off += TWF * Ns
        Ns *= R
        rem //= R
    assert off == len(tab)


def test_lengths_without_a_table_are_refused():
    from channel_rl_gb300.host import ChlError, fft_pass_table
    for N in (0, 5, 10, 14, 250):
        with pytest.raises(ChlError):
            fft_pass_table(N)
    assert len(fft_pass_table(4)) == 0 and len(fft_pass_table(2)) == 0
