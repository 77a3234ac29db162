"""Coder streams crafted for tests: a binary range encoder with the codec's
arithmetic, used to write payloads that no encoder of the codec would write."""


class RangeEncoder:
    """Binary range encoder with the codec's arithmetic (12-bit probabilities of
    a zero bit, shift-5 adaptation, bypass bits halve the range, five flush
    shifts; src/vc/vc.c:344-401). Used only to craft a payload that no
    encoder of the codec would write."""

    def __init__(self):
        self.low, self.range, self.cache, self.pending, self.out = 0, 0xFFFFFFFF, 0, 1, bytearray()

    def _shift(self):
        if (self.low & 0xFFFFFFFF) < 0xFF000000 or (self.low >> 32):
            carry, b = self.low >> 32, self.cache
            while True:
                self.out.append((b + carry) & 0xFF)
                b = 0xFF
                self.pending -= 1
                if not self.pending:
                    break
            self.cache = (self.low >> 24) & 0xFF
        self.pending += 1
        self.low = (self.low & 0x00FFFFFF) << 8

    def _norm(self):
        while self.range < (1 << 24):
            self._shift()
            self.range = (self.range << 8) & 0xFFFFFFFF

    def bit(self, ctx, i, b):
        r0 = (self.range * ctx[i]) >> 12
        if b:
            self.low += r0
            self.range -= r0
            ctx[i] -= ctx[i] >> 5
        else:
            self.range = r0
            ctx[i] += (4096 - ctx[i]) >> 5
        self._norm()

    def bypass(self, b):
        self.range >>= 1
        if b:
            self.low += self.range
        self._norm()

    def finish(self):
        for _ in range(5):
            self._shift()
        return bytes(self.out)


def hostile_payload(dc=100, prefix_ones=40):
    """[dc][coder bytes] of a stream whose first coefficient escapes with an
    exponential-Golomb prefix of `prefix_ones` ones: longer than any level can
    need, so a decoder must reject it as malformed."""
    e = RangeEncoder()
    sig, mag = [2048] * 8, [2048] * 12
    for i in range(15, -1, -1):   # EOB = 1
        e.bypass((1 >> i) & 1)
    e.bit(sig, 0, 1)              # scan position 0 (band 0) is significant
    for k in range(12):           # unary magnitude saturates, then the escape
        e.bit(mag, k, 1)
    for _ in range(prefix_ones):
        e.bypass(1)
    return bytes([dc]) + e.finish()
