"""Derives the constants used by nbg_math.h from first principles with mpmath.

Run `python gen_math_constants.py` to print them as C99 hex-float literals.

* Taylor coefficients of sin, cos and atan are 1/n! and (-1)^k/(2k+1),
  rounded to the nearest double.
* pi/2 is split Cody-Waite style (W. J. Cody, W. Waite, "Software Manual for
  the Elementary Functions", 1980): PIO2_1 and PIO2_2 keep 33 significant bits
  each so k*PIO2_1 and k*PIO2_2 are exact for |k| < 2^20, PIO2_3 is the rest.
* Other constants are the nearest double (and, for hi/lo pairs, the nearest
  double of the residual).
"""
import mpmath as mp

mp.mp.prec = 300


def hexd(v):
    return float(v).hex()


def trunc_bits(v, bits):
    # keep `bits` significant bits of v (truncate toward zero)
    m, e = mp.frexp(v)
    scale = mp.mpf(2) ** bits
    return mp.floor(m * scale) / scale * mp.mpf(2) ** e


def main():
    pio2 = mp.pi / 2
    p1 = trunc_bits(pio2, 33)
    p2 = trunc_bits(pio2 - p1, 33)
    p3 = mp.mpf(float(pio2 - p1 - p2))
    print("PIO2_1", hexd(p1))
    print("PIO2_2", hexd(p2))
    print("PIO2_3", hexd(p3))
    print("TWO_OVER_PI", hexd(2 / mp.pi))
    for name, v in (("PIO2", mp.pi / 2), ("PI", mp.pi), ("PIO6", mp.pi / 6),
                    ("PIO4", mp.pi / 4), ("PI3O4", 3 * mp.pi / 4)):
        hi = mp.mpf(float(v))
        lo = mp.mpf(float(v - hi))
        print(name + "_HI", hexd(hi), name + "_LO", hexd(lo))
    print("SQRT3", hexd(mp.sqrt(3)))
    print("TAN_PI_12", hexd(2 - mp.sqrt(3)))
    print("sin coefficients S1..S10 (x^3..x^21):")
    for k in range(1, 11):
        print("  ", hexd(mp.mpf(-1) ** k / mp.factorial(2 * k + 1)))
    print("cos coefficients C1..C11 (x^2..x^22):")
    for k in range(1, 12):
        print("  ", hexd(mp.mpf(-1) ** k / mp.factorial(2 * k)))
    print("atan coefficients A1..A14 (x^3..x^29):")
    for k in range(1, 15):
        print("  ", hexd(mp.mpf(-1) ** k / (2 * k + 1)))


if __name__ == "__main__":
    main()
