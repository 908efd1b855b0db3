"""The binomial checkpointing schedule of the window engine
(vardyn_gb300.fourdvar.revolve_schedule), simulated on the host: every unit
reversed exactly once and in reverse order, the snapshot stack within its
slots, and the recomputation count against the binomial bound
r*n - C(c+1+r-1, r-1) of Griewank and Walther (revolve), which the schedule
meets exactly when the split rule is tight."""
import math

import pytest

from vardyn_gb300.fourdvar import binomial_reach, revolve_schedule


def simulate(n, c):
    stack, cur, order, advances, peak = [], 0, [], 0, 0
    for act in revolve_schedule(n, c):
        kind = act[0]
        if kind == "advance":
            assert cur == act[1] and act[2] > act[1]
            advances += act[2] - act[1]
            cur = act[2]
        elif kind == "save":
            assert cur == act[1]
            stack.append(cur)
            peak = max(peak, len(stack))
        elif kind == "restore":
            assert stack and stack[-1] == act[1]
            cur = act[1]
        elif kind == "drop":
            assert stack.pop() == act[1]
        else:
            assert cur == act[1]
            order.append(act[1])
            cur = act[1] + 1
    assert not stack
    return order, advances, peak


@pytest.mark.parametrize("n,c", [(1, 0), (2, 0), (7, 0), (10, 2), (100, 5), (480, 20), (720, 40), (2880, 10)])
def test_schedule_reverses_every_unit_once_within_its_slots(n, c):
    order, advances, peak = simulate(n, c)
    assert order == list(range(n - 1, -1, -1))
    assert peak <= c + 1
    if c == 0:
        assert advances == n * (n - 1) // 2
    else:
        r = 1
        while binomial_reach(c, r) < n:
            r += 1
        bound = r * n - math.comb(c + r, r - 1)
        # within 12 % of the binomial optimum
        assert advances <= 1.12 * bound + 1


def test_schedule_is_optimal_where_the_split_is_tight():
    # n = 720 units, 40 slots: r = 2 and the optimum is 2 n - C(c + 2, 1) = 2 n - (c + 2)
    _, advances, _ = simulate(720, 40)
    assert advances == 2 * 720 - 42
