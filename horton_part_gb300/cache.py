"""Result cache and run-once methods with the reference's semantics.

``Cache`` stores keyed results with optional allocation and tags, and
``just_once`` makes a method run only on its first call and records its wall
time in ``time_usage`` (``core/cache.py:34-80``, ``core/cache.py:100-399`` in
horton-part). The partitioning classes of this package fill the same keys as
the reference (``charges``, ``propars``, ``niter``, ``history_*`` ...), so
code written against ``part.cache`` / ``part[key]`` works unchanged.
"""

from __future__ import annotations

import time

import numpy as np

__all__ = ["JustOnceClass", "just_once", "Cache"]


class JustOnceClass:
    """Base class whose ``@just_once`` methods run at most once until ``clear()``."""

    def __init__(self):
        self._done_just_once = set()
        self.time_usage = {}

    def __clear__(self):
        self.clear()

    def clear(self):
        self._done_just_once = set()


def just_once(fn):
    def wrapper(instance):
        if not hasattr(instance, "_done_just_once"):
            raise TypeError("Missing hidden _done_just_once. Forgot to call JustOnceClass.__init__()?")
        if fn.__name__ in instance._done_just_once:
            return
        t0 = time.time()
        fn(instance)
        t1 = time.time()
        instance._done_just_once.add(fn.__name__)
        instance.time_usage[fn.__name__] = t1 - t0

    wrapper.__doc__ = fn.__doc__
    wrapper.__name__ = fn.__name__
    return wrapper


def _norm_alloc(alloc):
    if not hasattr(alloc, "__len__"):
        alloc = (alloc,)
    if len(alloc) == 0:
        raise TypeError("Alloc can not be an empty list")
    return tuple(alloc)


def _norm_tags(tags):
    return set() if tags is None else set(tags)


def _norm_key(key):
    if hasattr(key, "__len__") and len(key) == 0:
        raise TypeError("At least one argument needed to specify a key.")
    while isinstance(key, tuple) and len(key) == 1:
        key = key[0]
    return key


class CacheItem:
    """A stored value with a validity flag and tags."""

    def __init__(self, value, tags=None):
        self._value = value
        self._valid = True
        self._tags = _norm_tags(tags)

    @classmethod
    def from_alloc(cls, alloc, tags):
        return cls(np.zeros(_norm_alloc(alloc), dtype=float), tags=tags)

    def check_alloc(self, alloc):
        alloc = _norm_alloc(alloc)
        v = self._value
        if not (isinstance(v, np.ndarray) and v.shape == alloc and issubclass(v.dtype.type, float)):
            raise TypeError("The stored item does not match the given alloc.")

    def check_tags(self, tags):
        if _norm_tags(tags) != self._tags:
            raise ValueError("Tags do not match.")

    @property
    def value(self):
        if not self._valid:
            raise ValueError("This cached item is not valid.")
        return self._value

    @property
    def valid(self):
        return self._valid

    @property
    def tags(self):
        return self._tags

    def clear(self):
        self._valid = False
        if isinstance(self._value, np.ndarray):
            self._value[:] = 0.0
        elif hasattr(self._value, "__clear__") and callable(self._value.__clear__):
            self._value.__clear__()
        else:
            return False
        return True


_no_default = object()


class Cache:
    """Dictionary-like store of previously computed results."""

    def __init__(self):
        self._store = {}

    def clear(self, **kwargs):
        dealloc = kwargs.pop("dealloc", False)
        tags = _norm_tags(kwargs.pop("tags", None))
        if kwargs:
            raise TypeError("Unexpected arguments: %s" % list(kwargs))
        for key, item in list(self._store.items()):
            if not tags or item.tags & tags:
                self.clear_item(key, dealloc=dealloc)

    def clear_item(self, *key, **kwargs):
        key = _norm_key(key)
        dealloc = kwargs.pop("dealloc", False)
        if kwargs:
            raise TypeError("Unexpected arguments: %s" % list(kwargs))
        item = self._store.get(key)
        if item is None:
            return
        if dealloc or not item.clear():
            del self._store[key]

    def load(self, *key, **kwargs):
        key = _norm_key(key)
        alloc = kwargs.pop("alloc", None)
        default = kwargs.pop("default", _no_default)
        tags = kwargs.pop("tags", None)
        if alloc is not None and default is not _no_default:
            raise TypeError("The optional arguments alloc and default can not be used at the same time.")
        if tags is not None and alloc is None:
            raise TypeError("The tags argument is only allowed when the alloc argument is present.")
        if kwargs:
            raise TypeError("Unknown optional arguments: %s" % list(kwargs))
        item = self._store.get(key)
        if alloc is not None:
            if item is None:
                item = CacheItem.from_alloc(alloc, tags)
                self._store[key] = item
                return item.value, True
            if not item.valid:
                try:
                    item.check_alloc(alloc)
                    item._valid = True
                    item.check_tags(tags)
                except TypeError:
                    item = CacheItem.from_alloc(alloc, tags)
                    self._store[key] = item
                return item.value, True
            item.check_alloc(alloc)
            item.check_tags(tags)
            return item.value, False
        if default is not _no_default:
            return default if item is None or not item.valid else item.value
        if item is None or not item.valid:
            raise KeyError(key)
        return item.value

    def __contains__(self, key):
        item = self._store.get(_norm_key(key))
        return item is not None and item.valid

    def dump(self, *args, **kwargs):
        tags = kwargs.pop("tags", None)
        if kwargs:
            raise TypeError("Unknown optional arguments: %s" % list(kwargs))
        if len(args) < 2:
            raise TypeError("At least two arguments are required: key1 and value.")
        self._store[_norm_key(args[:-1])] = CacheItem(args[-1], tags)

    def __len__(self):
        return sum(item.valid for item in self._store.values())

    def __getitem__(self, key):
        return self.load(key)

    def __setitem__(self, key, value):
        return self.dump(key, value)

    def __iter__(self):
        return iter(self.iterkeys())

    def iterkeys(self, tags=None):
        tags = _norm_tags(tags)
        for key, item in self._store.items():
            if item.valid and (not tags or item.tags & tags):
                yield key

    def itervalues(self, tags=None):
        tags = _norm_tags(tags)
        for item in self._store.values():
            if item.valid and (not tags or item.tags & tags):
                yield item.value

    def iteritems(self, tags=None):
        tags = _norm_tags(tags)
        for key, item in self._store.items():
            if item.valid and (not tags or item.tags & tags):
                yield key, item.value
