"""Keyed result store and run-once methods behind ``part.cache`` / ``part[key]``.

Callers of horton-part read results through ``part.cache`` (``load``,
``dump``, ``in``, ``iterkeys(tags="o")``, ``clear``) and rely on
``@just_once`` methods such as ``do_partitioning`` running at most once per
``clear()``; the interface is the one of horton-part's ``core/cache.py``.
This module is written from that behaviour (the acceptance list is the
reference's ``tests/core/test_cache.py``, restated in
``tests/test_cache_api.py``):

* keys are one or more hashable parts; ``c["a"]``, ``c[("a",)]`` and
  ``c.load("a")`` name the same entry, as do ``c["a", 1]`` and
  ``c.load("a", 1)``;
* ``load(key, alloc=shape)`` hands out a zero-filled float64 array the first
  time (returns ``(array, True)``) and the same array afterwards
  (``(array, False)``), checking its shape (``TypeError``) and tags
  (``ValueError``);
* clearing an entry that holds an array zero-fills the array and marks the
  entry stale, so a later ``alloc`` load with the same shape reuses the
  buffer; entries with a ``__clear__`` method are cleared through it; any
  other entry is removed;
* tags are sets of one-letter labels ("o" marks the scheme's outputs).
"""

from __future__ import annotations

import functools
import time

import numpy as np

__all__ = ["JustOnceClass", "just_once", "Cache"]


class JustOnceClass:
    """Base for classes with ``@just_once`` methods.

    The names of the methods that already ran sit in ``_done_just_once``;
    ``clear()`` forgets them. ``time_usage[name]`` holds the wall time of the
    last run of each such method.
    """

    def __init__(self):
        self._done_just_once = set()
        self.time_usage = {}

    def __clear__(self):
        self.clear()

    def clear(self):
        self._done_just_once = set()


def just_once(method):
    """Run ``method(self)`` only on its first call until ``self.clear()``."""
    name = method.__name__

    @functools.wraps(method)
    def run_once(self):
        done = getattr(self, "_done_just_once", None)
        if done is None:
            raise TypeError(f"{type(self).__name__}.{name} is @just_once, but the instance has no "
                            "run-once bookkeeping (JustOnceClass.__init__ was not called)")
        if name in done:
            return
        start = time.time()
        method(self)
        self._done_just_once.add(name)
        self.time_usage[name] = time.time() - start

    return run_once


_MISSING = object()


def _entry_key(parts):
    """One key from the positional parts of a call (nested 1-tuples unwrapped)."""
    if isinstance(parts, tuple) and len(parts) == 0:
        raise TypeError("a cache key needs at least one part")
    key = parts
    while isinstance(key, tuple) and len(key) == 1:
        key = key[0]
    return key


def _tag_set(tags):
    return frozenset(tags) if tags else frozenset()


def _shape_of(alloc):
    shape = tuple(alloc) if isinstance(alloc, (tuple, list)) else (alloc,)
    if not shape:
        raise TypeError("alloc must name at least one dimension")
    return shape


class _Entry:
    __slots__ = ("value", "stale", "tags")

    def __init__(self, value, tags):
        self.value = value
        self.stale = False
        self.tags = tags

    def holds_float_array(self, shape):
        v = self.value
        return isinstance(v, np.ndarray) and v.dtype == np.float64 and v.shape == shape

    def invalidate(self):
        """Reset the value in place; False when the entry cannot be kept."""
        v = self.value
        if isinstance(v, np.ndarray):
            v[...] = 0.0
        elif callable(getattr(v, "__clear__", None)):
            v.__clear__()
        else:
            return False
        self.stale = True
        return True


class Cache:
    """Store of computed results, keyed by one or more hashable parts."""

    def __init__(self):
        self._store = {}

    # -- reading ------------------------------------------------------------
    def _live(self, key):
        entry = self._store.get(key)
        return None if entry is None or entry.stale else entry

    def load(self, *key, alloc=None, default=_MISSING, tags=None):
        """Return the value under ``key``.

        ``default``: returned when the entry is absent or stale.
        ``alloc``: shape of a float64 array to hand out; returns
        ``(array, new)`` and creates (or revives) the entry when needed.
        ``tags`` may only accompany ``alloc``.
        """
        key = _entry_key(key)
        if alloc is not None and default is not _MISSING:
            raise TypeError("load takes either alloc or default, not both")
        if alloc is None:
            if tags is not None:
                raise TypeError("tags are given at allocation (or dump) time only")
            entry = self._live(key)
            if entry is not None:
                return entry.value
            if default is _MISSING:
                raise KeyError(key)
            return default
        return self._allocate(key, _shape_of(alloc), _tag_set(tags))

    def _allocate(self, key, shape, tags):
        entry = self._store.get(key)
        if entry is not None and entry.holds_float_array(shape):
            if entry.tags != tags:
                raise ValueError(f"cache entry {key!r} has tags {sorted(entry.tags)}, "
                                 f"not {sorted(tags)}")
            revived = entry.stale
            entry.stale = False
            return entry.value, revived
        if entry is not None and not entry.stale:
            raise TypeError(f"cache entry {key!r} is not a float array of shape {shape}")
        entry = _Entry(np.zeros(shape), tags)
        self._store[key] = entry
        return entry.value, True

    def __getitem__(self, key):
        return self.load(key)

    def __contains__(self, key):
        return self._live(_entry_key(key)) is not None

    def __len__(self):
        return sum(1 for e in self._store.values() if not e.stale)

    def _selected(self, tags):
        want = _tag_set(tags)
        for key, entry in self._store.items():
            if not entry.stale and (not want or entry.tags & want):
                yield key, entry.value

    def iterkeys(self, tags=None):
        return (k for k, _ in self._selected(tags))

    def itervalues(self, tags=None):
        return (v for _, v in self._selected(tags))

    def iteritems(self, tags=None):
        return self._selected(tags)

    def __iter__(self):
        return self.iterkeys()

    # -- writing ------------------------------------------------------------
    def dump(self, *key_and_value, tags=None):
        """``dump(key..., value, tags=None)``: store ``value`` under ``key``."""
        if len(key_and_value) < 2:
            raise TypeError("dump needs a key and a value")
        self._store[_entry_key(key_and_value[:-1])] = _Entry(key_and_value[-1], _tag_set(tags))

    def __setitem__(self, key, value):
        self.dump(key, value)

    def clear_item(self, *key, dealloc=False):
        """Invalidate (arrays, ``__clear__`` objects) or remove one entry."""
        key = _entry_key(key)
        entry = self._store.get(key)
        if entry is not None and (dealloc or not entry.invalidate()):
            del self._store[key]

    def clear(self, dealloc=False, tags=None):
        """Clear every entry, or those sharing a tag with ``tags``."""
        want = _tag_set(tags)
        for key in [k for k, e in self._store.items() if not want or e.tags & want]:
            self.clear_item(key, dealloc=dealloc)
