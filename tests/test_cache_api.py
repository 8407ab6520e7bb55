"""Behaviour of ``part.cache`` and ``@just_once`` that callers of horton-part rely on.

The cases restate the acceptance list of horton-part's ``tests/core/test_cache.py``
(key forms, allocation and reuse of cleared arrays, defaults, tags, dealloc,
iteration, argument errors) against this package's own ``Cache``, plus the
``Part``/``WPart`` host logic (populations and charges from cached
at_weights, grid types, geometry checks) without a GPU.
"""

import numpy as np
import pytest

from horton_part_gb300.cache import Cache, JustOnceClass, just_once
from horton_part_gb300.part import WPart
from horton_part_gb300.utils import typecheck_geo


class Counter(JustOnceClass):
    def __init__(self):
        super().__init__()
        self.count = 0

    @just_once
    def bump(self):
        self.count += 1

    def bump_always(self):
        self.count += 1


def test_just_once_runs_once_per_clear():
    c = Counter()
    c.bump()
    c.bump()
    assert c.count == 1 and "bump" in c.time_usage
    c.clear()
    c.bump()
    c.bump()
    assert c.count == 2
    c.bump_always()
    assert c.count == 3


def test_just_once_without_bookkeeping_is_a_type_error():
    class Bare:
        @just_once
        def f(self):
            pass

    with pytest.raises(TypeError):
        Bare().f()


@pytest.mark.parametrize("setter", ["dump", "item"])
def test_key_forms_name_one_entry(setter):
    c = Cache()
    if setter == "dump":
        c.dump("foo", 5)
        c.dump("foo", 4, 6)
    else:
        c["foo"] = 5
        c["foo", 4] = 6
    for got in (c["foo"], c[("foo",)], c.load("foo"), c.load(("foo",))):
        assert got == 5
    for got in (c["foo", 4], c[("foo", 4)], c.load("foo", 4), c.load(("foo", 4))):
        assert got == 6
    assert len(c) == 2
    c.clear()
    assert len(c._store) == 0 and len(c) == 0


@pytest.mark.parametrize("shape", [5, (5, 10)])
def test_alloc_hands_out_one_zeroed_array(shape):
    c = Cache()
    assert "bar" not in c
    a, new = c.load("bar", alloc=shape)
    assert new and a.shape == np.zeros(shape).shape and a.dtype == np.float64 and not a.any()
    assert "bar" in c
    a[3] = 1
    assert c.load("bar") is a
    b, new = c.load("bar", alloc=shape)
    assert not new and b is a


def test_cleared_array_is_reused_by_same_shape_only():
    c = Cache()
    a, _ = c.load("egg", alloc=(5, 10))
    with pytest.raises(TypeError):
        c.load("egg", alloc=10)
    with pytest.raises(TypeError):
        c.load("egg", alloc=(10, 5))
    a[:] = 1.0
    c.clear()
    assert "egg" not in c and not a.any()
    with pytest.raises(KeyError):
        c.load("egg")
    b, new = c.load("egg", alloc=(5, 10))
    assert new and b is a and "egg" in c and c.load("egg") is a
    c.clear()
    d, new = c.load("egg", alloc=(5, 1, 2))
    assert new and d.shape == (5, 1, 2) and d is not a


def test_multipart_keys():
    c = Cache()
    assert ("a", 1) not in c
    c.dump("a", 1, 2)
    assert ("a", 1) in c and c.load("a", 1) == 2
    c.dump(("foo",), 5)
    assert "foo" in c


def test_defaults():
    c = Cache()
    assert c.load("egg", default=5) == 5
    c.dump("egg", 5)
    assert c.load("egg", default=6) == 5
    c.clear()
    assert c.load("egg", default=6) == 6
    assert c.load("egg", default=None) is None
    with pytest.raises(KeyError):
        c.load("egg")
    c.dump("floep", np.array([3.1, 5.1]))
    assert (c.load("floep", default=3) == np.array([3.1, 5.1])).all()
    c.clear()
    assert c.load("floep", default=3) == 3


def test_argument_errors():
    c = Cache()
    with pytest.raises(KeyError):
        c.load("boo")
    c.dump("bar", np.zeros(4))
    with pytest.raises(TypeError):
        c.load("bar", alloc=5)
    for call in (lambda: c.load(), lambda: c.load("foo", sadfj=4),
                 lambda: c.load("foo", alloc=3, sdasffd=0), lambda: c.load("foo", alloc=3, default=0),
                 lambda: c.load("foo", jgfjg=3, default=0), lambda: c.dump(), lambda: c.dump("one"),
                 lambda: c.clear_item()):
        with pytest.raises(TypeError):
            call()


def test_dealloc_removes_entries():
    c = Cache()
    c.dump("foo", 5)
    c.dump("bar", 6)
    c.clear_item("foo", dealloc=True)
    assert "foo" not in c and "bar" in c and len(c._store) == 1
    c.dump("foo", 5)
    c.clear(dealloc=True)
    assert len(c._store) == 0


def test_iteration_and_tags():
    c = Cache()
    c.dump("foo", 5, tags="c")
    c.dump("bar", 6)
    c.dump("egg", 7, tags="op")
    c.dump("spam", 8, tags="co")
    assert sorted(c) == sorted(c.iterkeys()) == ["bar", "egg", "foo", "spam"]
    assert sorted(c.itervalues()) == [5, 6, 7, 8]
    assert sorted(c.iteritems()) == [("bar", 6), ("egg", 7), ("foo", 5), ("spam", 8)]
    assert sorted(c.iterkeys(tags="c")) == ["foo", "spam"]
    assert sorted(c.itervalues(tags="c")) == [5, 8]
    assert sorted(c.iteritems(tags="c")) == [("foo", 5), ("spam", 8)]
    assert list(c.iterkeys(tags="a")) == [] and len(c) == 4


def test_tags_are_fixed_at_allocation():
    c = Cache()
    c.dump("a", 5, tags="ab")
    for kw in ({"tags": "a"}, {"tags": "ab"}, {"tags": "abc"}):
        with pytest.raises(TypeError):
            c.load("a", **kw)
    with pytest.raises(TypeError):
        c.load("b", default=5, tags="abc")
    c.clear(tags="cd")
    assert len(c) == 1
    c.clear(tags="a")
    assert len(c) == 0
    t1, new = c.load("tmp", alloc=5, tags="qw")
    assert new
    t2, new = c.load("tmp", alloc=5, tags="qw")
    assert not new and t2 is t1
    for bad in ("w", "aw", "ab"):
        with pytest.raises(ValueError):
            c.load("tmp", alloc=5, tags=bad)
    c.clear()
    t3, new = c.load("tmp", alloc=5, tags="qw")
    assert new and t3 is t1
    with pytest.raises(ValueError):
        c.load("tmp", alloc=5, tags="w")


def test_typecheck_geo():
    xyz = np.zeros((2, 3))
    z = np.array([8, 1])
    natom, c, n, p = typecheck_geo(xyz, z, None)
    assert natom == 2 and p.dtype == np.float64 and (p == z).all()
    natom, p = typecheck_geo(None, None, np.array([6, 1]), need_coordinates=False, need_numbers=False)
    assert natom == 2 and p.dtype == np.float64
    for args in ((xyz, z.astype(np.int32)), (xyz.astype(np.float32), z), (np.zeros((3, 3)), z),
                 (xyz, z, np.zeros(3)), (None, z), (xyz, None)):
        with pytest.raises(TypeError):
            typecheck_geo(*args)
    with pytest.raises(TypeError):
        typecheck_geo()


class _Grid:
    """Two-point 'atomic grids' stacked into one molecular grid."""

    def __init__(self):
        self.points = np.array([[0.0, 0, 0], [1.0, 0, 0], [0, 2.0, 0], [0, 3.0, 0]])
        self.weights = np.array([1.0, 2.0, 3.0, 4.0])
        self.indices = np.array([0, 2, 4])
        self.atgrids = [_Sub(self.weights[:2]), _Sub(self.weights[2:])]

    def integrate(self, *arrays):
        return float(np.sum(self.weights * np.prod(arrays, axis=0)))


class _Sub:
    def __init__(self, w):
        self.weights = w

    def integrate(self, *arrays):
        return float(np.sum(self.weights * np.prod(arrays, axis=0)))


class _Fixed(WPart):
    """A scheme whose at_weights are given: checks the population bookkeeping."""

    def update_at_weights(self):
        self.cache.dump("at_weights_0", np.array([0.75, 0.5, 0.25, 0.0]))
        self.cache.dump("at_weights_1", np.array([0.25, 0.5, 0.75, 1.0]))


@pytest.mark.parametrize("grid_type", [1, 2, 3])
def test_populations_and_charges_from_at_weights(grid_type):
    g = _Grid()
    rho = np.array([1.0, 1.0, 0.5, 0.25])
    part = _Fixed(np.zeros((2, 3)), np.array([3, 1]), np.array([2.0, 1.0]), g, rho,
                  spindens=0.5 * rho, grid_type=grid_type)
    keys = part.do_all()
    w0, w1 = part["at_weights_0"], part["at_weights_1"]
    if grid_type != 3:  # local: each atom integrates on its own atomic grid
        exp0 = np.sum(g.weights[:2] * w0[:2] * rho[:2])
        exp1 = np.sum(g.weights[2:] * w1[2:] * rho[2:])
    else:
        exp0, exp1 = np.sum(g.weights * w0 * rho), np.sum(g.weights * w1 * rho)
    np.testing.assert_allclose(part["pseudo_populations"], [exp0, exp1])
    np.testing.assert_allclose(part["populations"], [exp0 + 1.0, exp1])
    np.testing.assert_allclose(part["charges"], [3 - exp0 - 1.0, 1 - exp1])
    np.testing.assert_allclose(part["spin_charges"], 0.5 * np.array([exp0, exp1]))
    assert {"charges", "populations", "pseudo_populations", "spin_charges"} <= set(keys)
    assert part.on_molgrid == (grid_type != 1) and part.local == (grid_type != 3)
    assert part.nelec == pytest.approx(g.integrate(rho))
    d = part.radial_distances
    np.testing.assert_allclose(d[0], np.linalg.norm(g.points, axis=1))
    part.clear()
    assert "charges" not in part.cache


def test_grid_type_checks():
    g = _Grid()
    rho = np.ones(4)
    with pytest.raises(AssertionError):
        _Fixed(np.zeros((2, 3)), np.array([3, 1]), None, g, rho, grid_type=4)
    g.atgrids = None
    with pytest.raises(ValueError):
        _Fixed(np.zeros((2, 3)), np.array([3, 1]), None, g, rho, grid_type=2)
    part = _Fixed(np.zeros((2, 3)), np.array([3, 1]), None, g, rho, grid_type=3)
    assert not part.local
