"""Generate the constant tables of avbd_crmath.cuh (run by hand; needs mpmath).

Prints C++ initialisers for:
  * the bits of 2/pi after the binary point, as 64-bit words (Payne-Hanek
    argument reduction of sin / cos);
  * pi/4, pi/2, pi and atan(k/4) (k = 1..4) as double-double (hi + lo);
  * the Taylor coefficients of sin ((-1)^n / (2n+1)!), cos ((-1)^n / (2n)!),
    asin ((2n)! / (4^n (n!)^2 (2n+1))) and atan ((-1)^n / (2n+1)), each as a
    double-double, so that the slow path can evaluate in double-double.

Usage: python gen_crmath_constants.py > /tmp/tables.txt
"""
import mpmath as mp

mp.mp.prec = 600


def dd(x):
    hi = float(x)
    lo = float(x - mp.mpf(hi))
    return hi, lo


def fmt(v):
    return float.hex(v)


def dd_list(name, vals):
    print(f"// {name}")
    for v in vals:
        hi, lo = dd(v)
        print(f"    {{{fmt(hi)}, {fmt(lo)}}},")


def main():
    two_over_pi = 2 / mp.pi
    words = []
    frac = two_over_pi
    for _ in range(8):
        frac *= 2**64
        w = int(mp.floor(frac))
        words.append(w)
        frac -= w
    print("// 2/pi, bits 1..512 after the binary point")
    print("    " + ", ".join(f"0x{w:016x}ull" for w in words))
    for name, v in (("pi/4", mp.pi / 4), ("pi/2", mp.pi / 2), ("pi", mp.pi)):
        hi, lo = dd(v)
        print(f"// {name}: {{{fmt(hi)}, {fmt(lo)}}}")
    dd_list("atan(k/4), k = 1..4", [mp.atan(mp.mpf(k) / 4) for k in range(1, 5)])
    dd_list("sin: (-1)^n / (2n+1)!, n = 1..15", [(-1) ** n / mp.factorial(2 * n + 1) for n in range(1, 16)])
    dd_list("cos: (-1)^n / (2n)!, n = 1..15", [(-1) ** n / mp.factorial(2 * n) for n in range(1, 16)])
    dd_list("asin: (2n)! / (4^n (n!)^2 (2n+1)), n = 1..56",
            [mp.factorial(2 * n) / (4**n * mp.factorial(n) ** 2 * (2 * n + 1)) for n in range(1, 57)])
    dd_list("atan: (-1)^n / (2n+1), n = 1..24", [mp.mpf((-1) ** n) / (2 * n + 1) for n in range(1, 25)])


if __name__ == "__main__":
    main()
