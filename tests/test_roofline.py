"""Roofline bookkeeping (CPU): the algorithmic bytes and flops bench.py divides
by measured times, and the sort pass count they assume."""
from stellarsolver_gb300 import roofline


def test_sort_passes_follow_the_size_rule():
    assert roofline.high_passes(1 << 20) == 3
    assert roofline.high_passes(1 << 21) == 3
    assert roofline.high_passes((1 << 21) + 1) == 4
    assert roofline.high_passes(1 << 24) == 4


def test_phase_bytes():
    n = 1 << 20
    mixed = roofline.phase_bytes(n, True)
    plain = roofline.phase_bytes(n, False)
    ref = roofline.phase_bytes(n, False, accuracy=False)
    # each radix pass and the fixup read and write a 12-byte (key, index) pair
    assert mixed["sort"] == 24 * n * 4
    assert roofline.phase_bytes(n, True, passes=4)["sort"] == 24 * n * 5
    # the reorder: 52 bytes per body, plus the hi/lo tails (MIXED) and
    # |a_old| with the walk-group cost (accuracy modes)
    assert ref["reorder"] == 52 * n
    assert plain["reorder"] == 68 * n
    assert mixed["reorder"] == 84 * n
    assert mixed["bbox"] == 8 * n and mixed["keys"] == 20 * n


def test_walk_flops():
    stats = {"interactions": 1000, "cell_interactions": 600}
    # the roofline counts 14 flops per interaction of either kind
    assert roofline.walk_flops(stats) == 14 * 1000
    # executed arithmetic: quadrupole cells at 33
    assert roofline.walk_flops_with_multipole(stats) == 14 * 400 + 33 * 600
