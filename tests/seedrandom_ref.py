"""A third, pure-Python restatement of the reference's random stream, for tests.

random@4.1.0's `Random.clone(seed)` seeds seedrandom@3.0.5 with String(seed)
and `float(min, max)` returns `next() * (max - min) + min`; seedrandom's
default generator is ARC4 (RC4-drop[256]) keyed by mixkey(seed).  Python
integers and floats reproduce the JavaScript arithmetic exactly here (every
intermediate is an integer below 2^61 or an exact power-of-two quotient).
"""


def mixkey(seed_text):
    units = seed_text.encode("utf-16-le")
    codes = [units[k] | (units[k + 1] << 8) for k in range(0, len(units), 2)]
    key = {}
    smear = 0
    for j, c in enumerate(codes):
        smear ^= key.get(j & 255, 0) * 19
        key[j & 255] = 255 & (smear + c)
    return [key[k] for k in range(len(key))]


class SeedRandom:
    def __init__(self, seed_text):
        key = mixkey(str(seed_text)) or [0]
        s = list(range(256))
        j = 0
        for i in range(256):
            t = s[i]
            j = (j + key[i % len(key)] + t) & 255
            s[i] = s[j]
            s[j] = t
        self.s, self.i, self.j = s, 0, 0
        self.g(256)

    def g(self, count):
        s, i, j, r = self.s, self.i, self.j, 0
        for _ in range(count):
            i = (i + 1) & 255
            t = s[i]
            j = (j + t) & 255
            s[i] = s[j]
            s[j] = t
            r = r * 256 + s[(s[i] + t) & 255]
        self.i, self.j = i, j
        return r

    def next(self):
        n, d, x = self.g(6), 2 ** 48, 0
        while n < 2 ** 52:
            n = (n + x) * 256
            d *= 256
            x = self.g(1)
        while n >= 2 ** 53:
            n //= 2
            d //= 2
            x >>= 1
        return (n + x) / d

    def float(self, mn, mx):
        return self.next() * (mx - mn) + mn
