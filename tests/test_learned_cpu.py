"""CPU checks of the warm-start tooling's host side: the seeded random decks
(splitmix64) and the deck lists of the comparison runs parse with the
library's deck reader, reproducibly."""
import tealeaf_cuda_gb300 as tl
from tealeaf_cuda_gb300 import learned


def test_deck_lists_parse():
    assert learned.parse_decks("standard,20000-20002,7") == ["standard", 20000, 20001, 20002, 7]
    assert learned.parse_decks("5") == [5]


def test_standard_and_random_decks_parse():
    std = tl.parse_deck(learned.deck_for("standard", 128, 3))
    assert (std.x_cells, std.y_cells, std.nstates, std.end_step) == (128, 128, 5, 3)
    assert std.states[0].density == 100.0 and std.states[1].energy == 25.0
    a = tl.parse_deck(learned.deck_for(20007, 64, 2))
    b = tl.parse_deck(learned.deck_for(20007, 64, 2))
    assert 4 <= a.nstates <= 9
    assert [a.states[k].density for k in range(a.nstates)] == [b.states[k].density for k in range(b.nstates)]
    c = tl.parse_deck(learned.deck_for(20008, 64, 2))
    assert [a.states[k].density for k in range(a.nstates)] != [c.states[k].density for k in range(c.nstates)]
