"""Host logic of the batch (pytorchsph_gb300.serve) that needs no GPU: the order of the
scenes in a batch and the force-pass groups over it."""
from pytorchsph_gb300.serve import force_groups, scene_order


def test_scene_order_groups_by_lanes_then_scheme_stably():
    lanes = [2, 1, 4, 1, 2, 1]
    schemes = [2, 2, 2, 1, 2, 2]
    order = scene_order(lanes, schemes)
    assert order == [3, 1, 5, 0, 4, 2]
    kinds = [(lanes[e], schemes[e]) for e in order]
    assert kinds == sorted(kinds)


def test_force_groups_tile_the_batch_in_runs():
    p_off = [0, 10, 25, 25, 40, 55]
    kinds = [(1, 1), (1, 2), (1, 2), (1, 2), (4, 2)]
    g = force_groups(p_off, kinds)
    assert g == [[0, 10, 1, 1], [10, 40, 1, 2], [40, 55, 4, 2]]
    assert g[0][0] == 0 and g[-1][1] == p_off[-1]
    assert all(a[1] == b[0] for a, b in zip(g, g[1:]))
    assert force_groups([0], []) == [[0, 0, 1, -1]]
