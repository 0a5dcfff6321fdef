"""The reference's seeded PRNG, for scene generation on the host.

Xorshift64 (core/src/math/rand.rs:118-183) and Uniform<f32>
(rand.rs:304-325), bit for bit.
"""
import numpy as np

MASK = (1 << 64) - 1
DEFAULT_SEED = 378682147834061  # rand.rs:121


class Xorshift64:
    def __init__(self, seed=DEFAULT_SEED):
        if seed == 0:
            raise ValueError("xorshift seed cannot be zero")
        self.x = seed & MASK

    def next_bits(self):
        x = self.x
        x ^= (x << 13) & MASK
        x ^= x >> 7
        x ^= (x << 17) & MASK
        self.x = x
        return x

    def uniform(self, start, end):
        """Uniform(start..end).sample(): a float in [1,2) minus one, scaled."""
        bits = (127 << 23) | (self.next_bits() >> 41)
        unit = np.float32(np.array([bits], np.uint32).view(np.float32)[0] - np.float32(1.0))
        return np.float32(np.float32(unit * np.float32(np.float32(end) - np.float32(start)))
                          + np.float32(start))
