"""The save / do schedules (nmag.when) against the expectations of the
reference's own tests of its when module (interface/nsim/test_when.py:
match and next time of every() with first/last, of & and of a | of &s).
CPU only."""
from nmag.when import at, every

CASES = [(2, 3, 22), (2, 3, 23), (3, 0, None)]


def test_every_match_with_first_and_last():
    for step, first, last in CASES:
        w = every("x", step, first=first, last=last)
        for x in range(40):
            expected = not (x < first or (last is not None and x > last)) and (x - first) % step == 0
            assert w.match_time({"x": x, "y": 0}) == expected, (step, first, last, x)


def test_every_next_with_first_and_last():
    for step, first, last in CASES:
        w = every("x", step, first=first, last=last)
        for x in range(40):
            expected = first if x < first else ((x - first) // step + 1) * step + first
            if last is not None and expected > last:
                expected = False
            got = w.next_time("x", {"x": x, "y": 0})
            assert got == expected and type(got) is type(expected), (step, first, last, x, got)


def test_and_match():
    w = every("x", 2) & every("y", 3)
    for x in range(10):
        for y in range(10):
            assert w.match_time({"x": x, "y": y}) == (x % 2 == 0 and y % 3 == 0)


def test_and_next():
    w = every("x", 2) & every("y", 3)
    for x in range(10):
        for y in range(10):
            expected = (y // 3 + 1) * 3 if x % 2 == 0 else False
            assert w.next_time("y", {"x": x, "y": y}) == expected, (x, y)


def test_or_of_ands_next():
    w = (at("x", 0) & every("y", 10)) | (every("x", 1, first=1) & every("y", 2))
    for x in range(4):
        for y in range(100):
            expected = (y // 10 + 1) * 10 if x == 0 else (y // 2 + 1) * 2
            assert w.next_time("y", {"x": x, "y": y}) == expected, (x, y)
