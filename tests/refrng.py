"""std::mt19937_64, restated from its published definition (Matsumoto and
Nishimura, 64-bit Mersenne Twister; the C++ standard fixes its parameters, so
every conforming std::mt19937_64 yields the same stream). The reference's
polynomial tests draw their inputs from std::mt19937_64(12345); this lets the
oracle be checked on exactly those inputs."""

_M64 = (1 << 64) - 1


class MT19937_64:
    n, m = 312, 156
    a = 0xB5026F5AA96619E9
    u, d = 29, 0x5555555555555555
    s, b = 17, 0x71D67FFFEDA60000
    t, c = 37, 0xFFF7EEE000000000
    l = 43
    f = 6364136223846793005
    upper = 0xFFFFFFFF80000000
    lower = 0x7FFFFFFF

    def __init__(self, seed=5489):
        self.mt = [0] * self.n
        self.mt[0] = seed & _M64
        for i in range(1, self.n):
            prev = self.mt[i - 1]
            self.mt[i] = (self.f * (prev ^ (prev >> 62)) + i) & _M64
        self.idx = self.n

    def _twist(self):
        mt = self.mt
        for i in range(self.n):
            x = (mt[i] & self.upper) | (mt[(i + 1) % self.n] & self.lower)
            xa = x >> 1
            if x & 1:
                xa ^= self.a
            mt[i] = mt[(i + self.m) % self.n] ^ xa
        self.idx = 0

    def __call__(self):
        if self.idx >= self.n:
            self._twist()
        y = self.mt[self.idx]
        self.idx += 1
        y ^= (y >> self.u) & self.d
        y ^= (y << self.s) & self.b
        y ^= (y << self.t) & self.c
        y ^= y >> self.l
        return y & _M64
