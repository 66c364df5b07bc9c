"""Storages, mirroring particular/src/storage.rs and `Between` (particular/src/lib.rs:300).

* Between(affected, affecting)        - lib.rs:296-300
* Ordered: affecting bodies first      - storage.rs:48-138
* Reordered: unordered + Ordered copy  - storage.rs:140-205

A compute method accepts any of them, as the blanket impls of storage.rs:207-241
turn them into Between(affected, affecting):
    &[P]         -> Between(slice, slice)
    &Ordered     -> Between(particles(), affecting())
    &Reordered   -> Between(unordered, affecting())
"""
import numpy as np

from .gravity import fields


class Between:
    """A pair of storages: the first is affected by the second."""

    __slots__ = ("affected", "affecting")

    def __init__(self, affected, affecting):
        self.affected = affected
        self.affecting = affecting

    def __iter__(self):
        yield self.affected
        yield self.affecting


def _default_is_affecting(packed):
    return packed[:, 3] != 0.0  # GravitationalField::is_affecting (gravity/mod.rs:29-34)


def _mask(particles, packed, is_affecting_fn):
    if is_affecting_fn is None:
        return _default_is_affecting(packed)
    if getattr(is_affecting_fn, "vectorized", False):
        return np.asarray(is_affecting_fn(packed), bool)
    if isinstance(particles, np.ndarray) and particles.dtype.names is None:
        rows = [tuple(r) for r in packed]
        return np.fromiter((bool(is_affecting_fn(r)) for r in rows), bool, len(rows))
    return np.fromiter((bool(is_affecting_fn(p)) for p in particles), bool, packed.shape[0])


class Ordered:
    """Particles with the affecting ones first; order inside each group is kept."""

    def __init__(self, packed, affecting_len):
        self._packed = packed
        self._affecting_len = int(affecting_len)

    @classmethod
    def new(cls, unordered, is_affecting_fn=None, dtype=np.float32):
        packed = fields(unordered, dtype)
        m = _mask(unordered, packed, is_affecting_fn)
        return cls(np.ascontiguousarray(np.concatenate([packed[m], packed[~m]])), int(m.sum()))

    @classmethod
    def with_groups(cls, affecting, non_affecting, is_affecting_fn=None, dtype=np.float32):
        """Ordered::with (storage.rs:61-80): affecting_len is the first non-affecting
        position of the concatenation."""
        packed = np.concatenate([fields(affecting, dtype), fields(non_affecting, dtype)])
        m = _mask(None, packed, is_affecting_fn)
        first = np.flatnonzero(~m)
        return cls(np.ascontiguousarray(packed), int(first[0]) if first.size else packed.shape[0])

    def affecting_len(self):
        return self._affecting_len

    def affecting(self):
        return self._packed[: self._affecting_len]

    def non_affecting(self):
        return self._packed[self._affecting_len:]

    def particles(self):
        return self._packed

    def as_between(self):
        return Between(self.particles(), self.affecting())


class Reordered:
    """The original particles plus an Ordered copy (storage.rs:140-205)."""

    def __init__(self, unordered, is_affecting_fn=None, dtype=np.float32):
        self.unordered = unordered
        self._unordered_packed = fields(unordered, dtype)
        self._ordered = Ordered.new(unordered, is_affecting_fn, dtype)

    def ordered(self):
        return self._ordered

    def affecting_len(self):
        return self._ordered.affecting_len()

    def affecting(self):
        return self._ordered.affecting()

    def non_affecting(self):
        return self._ordered.non_affecting()

    def reordered(self):
        return self._ordered.particles()

    def as_between(self):
        return Between(self._unordered_packed, self.affecting())


def as_between(storage):
    """The Between(affected, affecting) a storage stands for (storage.rs:207-241)."""
    if isinstance(storage, Between):
        return storage
    if isinstance(storage, (Ordered, Reordered)):
        return storage.as_between()
    return Between(storage, storage)
