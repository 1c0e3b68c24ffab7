"""float_set / vector_set against the expectations of the reference's own
tests of its sets module (interface/nsim/test_sets.py) and the examples of
its docstrings (sets.py:40-58,130-150).  CPU only."""
import pytest

from nmag import float_set, vector_set


def close(a, b):
    return len(a) == len(b) and all(abs(x - y) <= 1e-10 for x, y in zip(a, b))


@pytest.mark.parametrize("spec,expected", [
    ([0, 1, [], 9], list(range(10))),
    ([9, 8, [], 0], list(range(9, -1, -1))),
    ([9, 8, [], 0, 1, [], 9], list(range(9, 0, -1)) + list(range(10))),
    ([0, [9], 9], list(range(10))),
    ([9, [9], 0], list(range(9, -1, -1))),
])
def test_plain(spec, expected):
    assert float_set(spec) == expected


@pytest.mark.parametrize("spec,expected", [
    ([0, 0.1, [], 0.5], [0.0, 0.1, 0.2, 0.3, 0.4, 0.5]),
    ([0, 0.1, [], 0.45], [0.0, 0.1, 0.2, 0.3, 0.4, 0.45]),
    ([0, 0.1, [], 0.2], [0.0, 0.1, 0.2]),
    ([0, -0.1, [], -0.45], [0.0, -0.1, -0.2, -0.3, -0.4, -0.45]),
    ([0, 0.1, [], 0.5, 1, [], 3], [0.0, 0.1, 0.2, 0.3, 0.4, 0.5, 1.0, 1.5, 2.0, 2.5, 3.0]),
])
def test_suspensions(spec, expected):
    assert close(float_set(spec), expected)


def test_mixes():
    assert float_set([0, [3], 3, 4, [], 6]) == [0.0, 1.0, 2.0, 3.0, 4.0, 5.0, 6.0]
    assert close(float_set([0.05, 0.1, [], 1.0]), [0.05 * k for k in range(1, 21)])
    good = ([0.05 * k for k in range(1, 21)] + [1.0 + 0.1 * k for k in range(1, 11)]
            + [2.0 + 0.2 * k for k in range(1, 10)] + [3.8 + 0.02 * k for k in range(1, 21)]
            + [4.2 + 0.05 * k for k in range(1, 7)] + [4.5 + 0.1 * k for k in range(1, 6)]
            + [5.0 + 0.5 * k for k in range(1, 7)])
    spec = [0.05, 0.1, [], 1.0, 1.1, [], 2.0, 2.2, [], 3.8, 3.82, [], 4.2, 4.25, [], 4.5, 4.6, [],
            5.0, 5.5, [], 8.0]
    assert close(float_set(spec), good)
    assert float_set([0, 1, "...", 3]) == [0.0, 1.0, 2.0, 3.0]


def test_errors():
    for bad in ([1, [], 5], [0, 1, []], [0, [0], 5], [0, [2.5], 5], [0, 5, [], 1]):
        with pytest.raises(ValueError):
            float_set(bad)


def test_vector_set():
    assert vector_set([0, [4], 4], [1, 2, 3], normalize=False) == [
        [0.0, 0.0, 0.0], [1.0, 2.0, 3.0], [2.0, 4.0, 6.0], [3.0, 6.0, 9.0], [4.0, 8.0, 12.0]]
    v = vector_set([0, 1, [], 4], [1, 2, 3])
    assert close(v[1], [0.2672612419124244, 0.5345224838248488, 0.8017837257372732])
    assert close(v[4], [1.0690449676496976, 2.1380899352993952, 3.2071349029490928])
    assert vector_set([0, 2], [1, 2], normalize=False, units=3) == [[0.0, 0.0], [6.0, 12.0]]


def test_vectools():
    import nmag
    assert close(nmag.normalised_vector([3.0, 0.0, 4.0]), [0.6, 0.0, 0.8])
    assert nmag.vector3_dot([1, 2, 3], [4, 5, 6]) == 32
    assert nmag.vector3_cross([1, 0, 0], [0, 1, 0]) == (0, 0, 1)


def test_float_set_units_scale_all_but_the_n_step_range():
    # the reference's [a, [n], b] branch appends its values without units
    # (interface/nsim/sets.py:88-97); its other branches scale them
    assert float_set([1, 2, [], 4], units=10) == [10.0, 20.0, 30.0, 40.0]
    assert float_set([1, [3], 4], units=10) == [10.0, 2.0, 3.0, 4.0]
