"""CPU check of the index algebra of the prime-factor row transforms
(aeolus_gb300/csrc/rows_pfa.cuh): n = R0 x R1 x R2 with the spectrum map
spec(q) = ((P^-1 q) mod R0) P + sw(R2 (n2 mod R1) + n2 div R1),
n2 = (R0^-1 q) mod P, the grid map grid(i) = (i mod R0) P + sw(i mod P), and
sw(u) = (u & ~7) | ((u ^ (u >> 3)) & 7) the XOR swizzle inside each P-point
block.  The passes below visit positions exactly as pfa_pass does (radix R2
over sw(8k + t), radix R1 over sw(8t + k) with the twiddles w_P^(k t)), so the
complex n-point transforms they compose must equal the DFT.  Exact complex
arithmetic here; the kernels do the same steps in 64-bit fixed point.
"""
import numpy as np
import pytest

SHAPES = [(3, 8, 8), (5, 4, 8), (3, 4, 8), (1, 8, 8), (1, 4, 8)]  # nlon 384, 320, 192, 128, 64


def sw(u):
    return (u & ~7) | ((u ^ (u >> 3)) & 7)


def inv_mod(a, m):
    return next(x for x in range(m) if (a * x) % m == 1 % m)


def maps(R0, R1, R2):
    P = R1 * R2
    n = R0 * P
    Pinv, R0inv = inv_mod(P, R0), inv_mod(R0, P)

    def upos(q):
        n2 = (R0inv * q) % P
        return sw(R2 * (n2 % R1) + n2 // R1)

    spec = np.array([((Pinv * q) % R0) * P + upos(q) for q in range(n)])
    grid = np.array([(i % R0) * P + sw(i % P) for i in range(n)])
    return P, n, spec, grid


def dft(v, sign):
    m = len(v)
    k = np.arange(m)
    return np.exp(sign * 2j * np.pi * np.outer(k, k) / m) @ v


def p_point(buf, R0, R1, R2, sign):
    """The two radix passes of every P-point block, in the order of the
    kernel's inverse (sign +1: radix R2 then twiddled radix R1) or forward
    (sign -1: twiddled radix R1 then radix R2) transform."""
    P = R1 * R2
    for r in range(R0):
        b = buf[r * P:(r + 1) * P]

        def pass1():
            for k in range(R1):
                pos = [sw(8 * k + t) for t in range(R2)]
                b[pos] = dft(b[pos], sign)

        def pass2():
            for k in range(R2):
                pos = [sw(8 * t + k) for t in range(R1)]
                w = np.exp(sign * 2j * np.pi * k * np.arange(R1) / P)
                b[pos] = dft(b[pos] * w, sign) if sign > 0 else dft(b[pos], sign) * w

        for f in ((pass1, pass2) if sign > 0 else (pass2, pass1)):
            f()


def radix_r0(buf, R0, P, sign):
    if R0 == 1:
        return
    for u in range(P):
        pos = [r * P + u for r in range(R0)]
        buf[pos] = dft(buf[pos], sign)


@pytest.mark.parametrize("R0,R1,R2", SHAPES)
def test_maps_are_permutations(R0, R1, R2):
    P, n, spec, grid = maps(R0, R1, R2)
    assert sorted(spec) == list(range(n))
    assert sorted(grid) == list(range(n))
    assert max(spec) < 2 ** 16 and max(grid) < 2 ** 16  # the kernels tabulate them as 16-bit words


@pytest.mark.parametrize("R0,R1,R2", SHAPES)
def test_inverse_and_forward_compose_the_dft(R0, R1, R2):
    P, n, spec, grid = maps(R0, R1, R2)
    rng = np.random.default_rng(R0 * 100 + R1)
    z = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    # inverse: spectrum map in, radix-R0 across the blocks, P-point blocks, grid map out
    buf = np.zeros(n, complex)
    buf[spec] = z
    radix_r0(buf, R0, P, +1)
    p_point(buf, R0, R1, R2, +1)
    x = buf[grid]
    np.testing.assert_allclose(x, np.fft.ifft(z) * n, rtol=0, atol=1e-9 * np.abs(z).sum())
    # forward: grid map in, P-point blocks, radix-R0 across the blocks, spectrum map out
    buf = np.zeros(n, complex)
    buf[grid] = x
    p_point(buf, R0, R1, R2, -1)
    radix_r0(buf, R0, P, -1)
    np.testing.assert_allclose(buf[spec], z * n, rtol=0, atol=1e-9 * n * np.abs(z).sum())
