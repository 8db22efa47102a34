"""Host logic of the batched solvers that needs no GPU: the stream priority levels of the
concurrent groups and the problem draw."""

from sfem_gb300.batch import draw_problems, stream_priority_levels


def test_stream_priority_levels():
    # smallest group on the top level, largest on level 0, levels monotone in size
    sizes = [500, 10, 70, 3000, 10, 800, 45, 1200]
    lv = stream_priority_levels(sizes, levels=6)
    assert lv[sizes.index(3000)] == 0 and max(lv) == 5 == lv[1]
    order = sorted(range(len(sizes)), key=lambda i: sizes[i])
    assert all(lv[a] >= lv[b] for a, b in zip(order, order[1:]))
    # fewer groups than levels: the smallest still on the top level, the largest on 0
    assert stream_priority_levels([3, 1, 2], levels=6) == [0, 5, 3]
    assert stream_priority_levels([7]) == [0] and stream_priority_levels([]) == []


def test_draw_problems_is_seeded_and_uneven():
    a, b = draw_problems(64, seed=3), draw_problems(64, seed=3)
    assert a == b and draw_problems(64, seed=4) != a
    assert {p.kind for p in a} == {"poisson", "elasticity"} and len({p.n for p in a}) > 4
    assert all(p.level in (2, 3, 4) and 8 <= p.n <= 32 for p in a)
