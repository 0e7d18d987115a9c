"""Prints the binary expansion of 2/pi as 32-bit words and the three-float
split of pi/2 used by the trigonometric range reductions in nt2g_math.cuh.

pi comes from Machin's formula, pi = 16 atan(1/5) - 4 atan(1/239), evaluated
in exact integer arithmetic with guard bits; 2/pi is then floor(2^K * 2/pi).
"""
import struct
import sys


def pi_fixed(bits):
    """floor(pi * 2^bits), exact (the guard bits absorb the series truncation)."""
    g = bits + 64
    one = 1 << g

    def atan_inv(q):  # atan(1/q) * 2^g by its alternating series
        s, term, k, q2 = 0, one // q, 0, q * q
        while term:
            s += term // (2 * k + 1) if k % 2 == 0 else -(term // (2 * k + 1))
            term //= q2
            k += 1
        return s

    return (16 * atan_inv(5) - 4 * atan_inv(239)) >> 64


def twoopi_words(nwords, guard=64):
    bits = 32 * nwords
    p = pi_fixed(bits + guard)  # pi * 2^(bits+guard)
    v = (1 << (2 * (bits + guard) + 1)) // p  # floor(2/pi * 2^(bits+guard))
    v >>= guard
    return [(v >> (32 * (nwords - 1 - i))) & 0xFFFFFFFF for i in range(nwords)]


def f32(x):
    return struct.unpack("<f", struct.pack("<f", x))[0]


def pio2_split():
    """C1 + C2 + C3 ~ pi/2 with each term the float nearest the remainder."""
    from fractions import Fraction
    pio2 = Fraction(pi_fixed(200), 1 << 201)
    out, rem = [], pio2
    for _ in range(3):
        c = f32(float(rem))
        out.append(c)
        rem -= Fraction(c)
    return out


if __name__ == "__main__":
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 8
    print(", ".join(f"0x{w:08X}u" for w in twoopi_words(n)))
    for c in pio2_split():
        print(f"{c.hex()}  0x{struct.unpack('<I', struct.pack('<f', c))[0]:08x}")
