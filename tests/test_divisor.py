"""Division by an invariant divisor as the Monte-Carlo kernels apply it
(Granlund & Montgomery, PLDI 1994, fig. 4.1), restated here: the kernels map
a unit to its (burst, sample) by dividing by the samples per burst, and bin a
unit's acceptor count by dividing by the burst's photon count, with a
multiplier and shift computed once per divisor."""
import numpy as np


def _divisor_of(d):
    """Granlund & Montgomery (PLDI 1994, fig. 4.1) as the kernels apply it:
    multiplier and shift of an invariant divisor 1 <= d < 2^31."""
    l = (d - 1).bit_length() if d > 1 else 0
    m = (((1 << l) - d) << 32) // d + 1
    return m & 0xFFFFFFFF, l


def _div_by(n, m, l):
    t = (m * n) >> 32
    return (t + ((n - t) >> min(l, 1))) >> max(l - 1, 0)


def test_invariant_divisor_quotients_are_exact():
    """The kernels' unit -> (burst, sample) and bin divisions: exact for every
    32-bit numerator (checked at the edges and at random) for the divisors the
    path uses (samples per burst, photons per burst up to 2^21) and beyond."""
    rng = np.random.default_rng(7)
    divisors = list(range(1, 2050)) + [2 ** k + e for k in range(11, 31) for e in (-1, 0, 1)]
    divisors += [int(x) for x in rng.integers(1, 2 ** 31, 500)]
    for d in divisors:
        m, l = _divisor_of(d)
        ns = [0, 1, d - 1, d, d + 1, 2 ** 31 - 1, 2 ** 32 - 1, (2 ** 32 - 1) // d * d,
              (2 ** 32 - 1) // d * d - 1] + [int(x) for x in rng.integers(0, 2 ** 32, 64)]
        for n in ns:
            if 0 <= n < 2 ** 32:
                assert _div_by(n, m, l) == n // d, (n, d)
