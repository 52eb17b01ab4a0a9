"""Growable structure-of-arrays storage used by the particle and node containers.

Woo keeps every particle and node as a heap object behind ``shared_ptr``
(pkg/dem/Particle.hpp:26-123, core/Field.hpp:50-108). Here the host keeps the
same data as contiguous numpy columns, which is also the layout the device
kernels consume, so uploading a scene is a handful of bulk copies.
"""
import numpy as np


class SoA:
    """A set of equally long numpy columns with amortised append."""

    def __init__(self, spec):
        # spec: name -> (dtype, trailing shape tuple, fill value)
        self._spec = dict(spec)
        self._n = 0
        self._cap = 0
        self._cols = {k: np.empty((0,) + tuple(sh), dtype=dt) for k, (dt, sh, _) in self._spec.items()}

    def __len__(self):
        return self._n

    def _grow(self, need):
        if need <= self._cap:
            return
        cap = max(need, 2 * self._cap, 16)
        for k, (dt, sh, fill) in self._spec.items():
            new = np.empty((cap,) + tuple(sh), dtype=dt)
            new[: self._n] = self._cols[k][: self._n]
            new[self._n:] = fill
            self._cols[k] = new
        self._cap = cap

    def append(self, count, **values):
        """Append ``count`` rows; columns not given take their fill value. Returns the first index."""
        start = self._n
        self._grow(start + count)
        for k, v in values.items():
            self._cols[k][start: start + count] = v
        self._n = start + count
        return start

    def col(self, name):
        """Live view of the used part of a column."""
        return self._cols[name][: self._n]

    def clear(self):
        self._n = 0
