"""Big-integer model of the Helios/Selene cycle -- TEST INFRASTRUCTURE ONLY.

This module is part of the oracle: only the test suite, the smoke check and
the CPU-baseline leg of the benchmark may import it.  It is a plain
mathematical restatement (Python ints, affine coordinates) used to
cross-check the C oracle (hs_oracle.c) on small inputs; it is far too slow
for anything else.

Reference behaviour restated here (helioselene sources):
  * curve equations y^2 = x^3 - 3x + b, generators and orders:
    helios/include/helios_constants.h:36-64, selene/include/selene_constants.h:36-64
  * q = 2^255 - gamma: fq/include/x64/fq51.h:38-62
  * point encoding (x little-endian, y parity in bit 255, identity = 32 zero
    bytes): helios/src/x64/helios_tobytes.cpp:42-66
  * decoding (mask bit 255, reject x >= p, sqrt, parity fix):
    helios/src/x64/helios_frombytes.cpp:59-109
  * simplified SWU map (RFC 9380 6.6.2, Z=7 on Helios, Z=-4 on Selene,
    sgn0(y) := sgn0(u)): helios/src/x64/helios_map_to_curve.cpp:98-198,
    selene/src/x64/selene_map_to_curve.cpp
"""

P = 2**255 - 19
GAMMA = 85737960593035654572250192257530476641
Q = 2**255 - GAMMA


class Curve:
    def __init__(self, name, field, order, b, gx, sswu_z):
        self.name = name
        self.F = field          # coordinate field modulus
        self.order = order      # prime group order (the other field)
        self.b = b
        self.gx = gx
        self.z = sswu_z % field
        self.gy = self._lift(gx, 0)

    # ---- field helpers ----
    def sqrt(self, a):
        F = self.F
        a %= F
        if a == 0:
            return 0
        if F % 4 == 3:
            r = pow(a, (F + 1) // 4, F)
        else:  # F = 5 mod 8
            r = pow(a, (F + 3) // 8, F)
            if r * r % F != a:
                r = r * pow(2, (F - 1) // 4, F) % F
        return r if r * r % F == a else None

    def _lift(self, x, parity):
        y = self.sqrt(x**3 - 3 * x + self.b)
        if y is None:
            return None
        if (y & 1) != parity:
            y = (-y) % self.F
        return y

    def on_curve(self, pt):
        if pt is None:
            return True
        x, y = pt
        return (y * y - (x**3 - 3 * x + self.b)) % self.F == 0

    # ---- group law (affine, None = identity) ----
    def add(self, a, b):
        F = self.F
        if a is None:
            return b
        if b is None:
            return a
        x1, y1 = a
        x2, y2 = b
        if x1 == x2:
            if (y1 + y2) % F == 0:
                return None
            lam = (3 * x1 * x1 - 3) * pow(2 * y1, -1, F) % F
        else:
            lam = (y2 - y1) * pow(x2 - x1, -1, F) % F
        x3 = (lam * lam - x1 - x2) % F
        return (x3, (lam * (x1 - x3) - y1) % F)

    def neg(self, a):
        return None if a is None else (a[0], (-a[1]) % self.F)

    def mul(self, k, pt):
        r = None
        for bit in bin(k)[2:] if k > 0 else "":
            r = self.add(r, r)
            if bit == "1":
                r = self.add(r, pt)
        return r

    def msm(self, scalars, points):
        """Sum of s_i * P_i for arbitrary 256-bit s_i (the mathematically correct MSM)."""
        acc = None
        for s, pt in zip(scalars, points):
            acc = self.add(acc, self.mul(s % self.order, pt))
        return acc

    # ---- encoding ----
    def encode(self, pt):
        if pt is None:
            return bytes(32)
        x, y = pt
        return (x | ((y & 1) << 255)).to_bytes(32, "little")

    def decode(self, data):
        v = int.from_bytes(data, "little")
        parity = v >> 255
        x = v & ((1 << 255) - 1)
        if x >= self.F:
            return "invalid"
        y = self._lift(x, parity)
        return "invalid" if y is None else (x, y)

    # ---- simplified SWU ----
    def map_to_curve(self, u_bytes):
        F = self.F
        u = (int.from_bytes(u_bytes, "little") & ((1 << 255) - 1)) % F
        A, B, Z = F - 3, self.b, self.z
        tv = (Z * Z * pow(u, 4, F) + Z * u * u) % F
        if tv == 0:
            x1 = B * pow(Z * A, -1, F) % F
        else:
            x1 = (-B) * pow(A, -1, F) * (1 + pow(tv, -1, F)) % F
        gx1 = (x1**3 + A * x1 + B) % F
        y1 = self.sqrt(gx1)
        if y1 is not None:
            x, y = x1, y1
        else:
            x = Z * u * u * x1 % F
            y = self.sqrt(x**3 + A * x + B)
        if (u & 1) != (y & 1):
            y = (-y) % F
        return (x, y)


HELIOS = Curve(
    "helios", P, Q,
    15789920373731020205926570676277057129217619222203920395806844808978996083412,
    3, 7)
SELENE = Curve(
    "selene", Q, P,
    50691664119640283727448954162351551669994268339720539671652090628799494505816,
    1, -4)
CURVES = {"helios": HELIOS, "selene": SELENE}
