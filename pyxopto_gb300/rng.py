"""Seeds of the per-thread multiply-with-carry random number streams
(the reference's xopto/cl/clrng.py Random: seeds(), initializer())."""
import numpy as np

from . import _lib


class Random:
    """Random(...).seeds(n, xinit) -> (x uint64[n], a uint32[n]).

    The multipliers are the safe-prime table of the reference
    (xopto/data/primes/safeprimes_base32_500k.npz), computed by the library
    on demand; the seed expansion is the reference's init_RNG."""
    MAXSEEDS = 1 << 22

    def __init__(self):
        self._lib = _lib.load()

    maxseeds = property(lambda self: self.MAXSEEDS)

    def multipliers(self, n: int) -> np.ndarray:
        a = np.zeros((int(n),), dtype=np.uint32)
        _lib.check(self._lib.mcgb_rng_safeprimes(a.ctypes.data, int(n)))
        return a

    def initializer(self, rng: np.random.Generator = None) -> int:
        """A random valid 64-bit initializer (clrng.py:446-462)."""
        first = int(self.multipliers(1)[0])
        rng = rng or np.random.default_rng()
        while True:
            xinit = int(rng.integers(1, 2 ** 64 - 1, dtype=np.uint64))
            if not (xinit == 0 or (xinit >> 32) >= first - 1 or (xinit & 0xFFFFFFFF) >= 0xFFFFFFFF):
                return xinit

    def seeds(self, n: int, xinit: int = None):
        n = int(n)
        if n < 0 or n > self.MAXSEEDS:
            raise ValueError('Cannot generate more than {} seeds, requested {}!'.format(self.MAXSEEDS, n))
        reinit = xinit is None
        if reinit:
            xinit = self.initializer()
        while True:
            x = np.zeros((n,), dtype=np.uint64)
            a = np.zeros((n,), dtype=np.uint32)
            r = self._lib.mcgb_rng_init(x.ctypes.data, a.ctypes.data, n, int(np.uint64(xinit)))
            if r == 0:
                return x, a
            if not reinit:
                raise ValueError('The provided initializer {} is not valid. Try a different '
                                 '64-bit unsigned integer!'.format(xinit))
            xinit = self.initializer()
