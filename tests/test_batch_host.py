"""CPU: the batch autotuner's choice rule (no GPU: times are given)."""
from __future__ import annotations

from phylocaml_gb300 import batch as B


def test_ties_go_to_the_first_candidate():
    c = B.CANDIDATES
    assert c[0] == B.Options(True, "cost")
    times = {o: 100.0 for o in c}
    times[B.Options(True, "variant")] = 99.0          # 1 % faster: a tie
    assert B.pick(times) == B.Options(True, "cost")
    times[B.Options(True, "variant")] = 90.0          # 10 % faster: it wins
    assert B.pick(times) == B.Options(True, "variant")
    times = {o: 100.0 for o in c}
    times[B.Options(False, "cost")] = 60.0
    assert B.pick(times) == B.Options(False, "cost")
