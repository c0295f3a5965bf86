"""The autotuner's choice of one node layout for a whole frame (host logic,
no GPU)."""
from bvhraytracer_gb300.autotune import one_layout

A, B = ("fp32", 0), ("fp32", 2)
O1, O2 = (("scheme", "per_ray"),), (("scheme", "persistent"),)


def _table(rows):
    return {(bi, lay, opts): ms for bi, lay, opts, ms in rows}


def test_one_layout_when_mixing_saves_little():
    # Batch 0 is 1 % faster in B, batch 1 only runs well in A: the frame in A
    # costs 1.02 against 1.01 mixed, within 3 %.
    t = _table([(0, A, O1, 0.51), (0, B, O1, 0.50), (1, A, O2, 0.51), (1, B, O2, 0.60)])
    assert one_layout(t, 2, mixed_ms=1.01) == A


def test_mixed_layouts_kept_when_they_save_more_than_the_margin():
    t = _table([(0, A, O1, 1.00), (0, B, O1, 0.50), (1, A, O2, 0.50), (1, B, O2, 1.00)])
    assert one_layout(t, 2, mixed_ms=1.00) is None
    assert one_layout(t, 2, mixed_ms=1.00, margin=0.6) in (A, B)


def test_layout_missing_a_batch_is_not_chosen():
    # B has no candidate for batch 1 (e.g. a stream-only option on Q8 nodes).
    t = _table([(0, A, O1, 0.60), (0, B, O1, 0.10), (1, A, O2, 0.50)])
    assert one_layout(t, 2, mixed_ms=0.60) is None  # A costs 1.10
    assert one_layout(t, 2, mixed_ms=1.10) == A


def test_best_option_per_batch_counts():
    t = _table([(0, A, O1, 0.90), (0, A, O2, 0.40), (1, A, O1, 0.30), (1, B, O1, 0.29),
                (0, B, O1, 0.41)])
    # A: 0.40 + 0.30 = 0.70; B: 0.41 + 0.29 = 0.70: either is within 3 % of 0.69.
    assert one_layout(t, 2, mixed_ms=0.69) in (A, B)
