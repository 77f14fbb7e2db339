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


def test_composition_key_groups_equal_mixes():
    """The autotuner's cache key: the (states x rate classes) mix and the
    pattern-count octiles, so batches with the same make-up share a choice."""
    import numpy as np
    from phylocaml_gb300 import mlmodel as M, synth, tree as T

    def var(S, R, n_pat):
        q, pi = (synth.protein_model(np.random.default_rng(S)) if S == 20
                 else synth.codon_model(2.0, 0.5))
        rates = M.gamma_rates(0.5, R) if R > 1 else np.ones(1)
        return B.Variant(T.yule(8, np.random.default_rng(1), 0.1), q, pi, rates, np.full(R, 1.0 / R),
                         synth.state_code_table(S), None, None, n_pat)

    a = [var(20, 4, 1000), var(61, 1, 5000)] * 4
    b = [var(61, 1, 5100), var(20, 4, 1010)] * 4          # same mix, counts in the same octiles
    c = [var(20, 4, 1000)] * 8                             # another mix
    assert B.composition_key(a) == B.composition_key(b)
    assert B.composition_key(a) != B.composition_key(c)
    assert "20x4:0.5" in B.composition_key(a) and "61x1:0.5" in B.composition_key(a)
    assert B.ORDERS == {"variant": 0, "cost": 1}
