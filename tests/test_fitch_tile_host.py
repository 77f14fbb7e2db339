"""CPU: the Fitch tree kernel's launch-shape model (fitch.tile_candidates,
fitch.default_tile), which ranks tile widths by the words the busiest SM
handles when all CTAs are resident."""
from __future__ import annotations

import pytest

from phylocaml_gb300 import fitch


def busiest(n_words: int, n_sm: int, w: int) -> int:
    tiles = -(-n_words // w)
    return -(-tiles // n_sm) * w


@pytest.mark.parametrize("n_words", [1, 626, 2_502, 25_000, 125_000, 1_000_000])
@pytest.mark.parametrize("n_sm", [132, 148, 152])
def test_default_tile_is_the_cheapest_wide_width(n_words, n_sm):
    w = fitch.default_tile(n_words, n_sm)
    assert 128 <= w <= 256 and w % 4 == 0
    cost = busiest(n_words, n_sm, w)
    for other in range(128, 257, 4):
        c = busiest(n_words, n_sm, other)
        # no width is cheaper, and a tie keeps the narrower width
        assert c > cost or (c == cost and other >= w)


def test_default_tile_at_the_benchmark_size():
    # 1e6 sites at 4-bit lanes: 601 CTAs of 208 words, 4 on the busiest SM
    assert fitch.default_tile(125_000, 152) == 208
    assert busiest(125_000, 152, 208) == 832 < busiest(125_000, 152, 128) == 896


def test_small_alignments_keep_narrow_tiles():
    # every width fits one wave: the narrowest keeps the most CTAs
    assert fitch.default_tile(626, 152) == 128


@pytest.mark.parametrize("n_words", [2_502, 125_000])
def test_candidates(n_words):
    c = fitch.tile_candidates(n_words, 152)
    assert 128 in c and fitch.default_tile(n_words, 152) in c
    assert all(64 <= w <= 256 and w % 4 == 0 for w in c)
    costs = [busiest(n_words, 152, w) for w in c]
    assert costs == sorted(costs)
