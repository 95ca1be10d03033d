"""Chunk planning of the NeRF MLP's recomputation mode (host logic, no GPU):
chunks hold whole rays, start at 512-byte-aligned row offsets, and each chunk's
backward workspace fits the activation budget."""
import pytest

from simple_rf_gb300.functional import recompute_rows


def _ws(rows):
    # the shape of the real workspace size: a fixed part (packed weights) + per-row activations
    return 1_200_000 + 4_700 * rows


def test_everything_fits_means_no_recomputation():
    assert recompute_rows(4096 * 192, 192, _ws(4096 * 192), _ws) == 0
    assert recompute_rows(0, 192, 1, _ws) == 0


@pytest.mark.parametrize('m,div,budget', [(4096 * 192, 192, 1 << 30), (65536 * 64, 64, 3 << 30),
                                          (1000, 1, 2_000_000), (777 * 260, 260, 100_000_000)])
def test_chunks_are_whole_rays_within_budget(m, div, budget):
    rows = recompute_rows(m, div, budget, _ws)
    assert rows > 0 and rows % div == 0 and rows % 128 == 0
    assert _ws(rows) <= budget
    # the largest such chunk: one more unit would not fit (or would cover every row)
    unit = div * 128 // __import__('math').gcd(div, 128)
    assert _ws(rows + unit) > budget or rows + unit >= m + unit


def test_budget_below_one_unit_raises():
    with pytest.raises(RuntimeError, match='activation budget'):
        recompute_rows(4096 * 192, 192, _ws(384) - 1, _ws)


def test_tensorf_graph_step_capacities():
    """Capacities of the captured TensoRF step: above every count by the margin,
    multiples of 1024 rows, and growing by the re-capture margin after an overflow."""
    from simple_rf_gb300.tensorf_step import TensorfGraphStep as G
    caps = G.capacities([(2349211, 1141923), (581631, 288894), (0, 0)], G.MARGIN)
    for (v, s), (cv, cs) in zip([(2349211, 1141923), (581631, 288894), (0, 0)], caps):
        assert cv % G.ROUND == 0 and cs % G.ROUND == 0
        assert cv > v * G.MARGIN and cs > s * G.MARGIN
        assert cv - v * G.MARGIN <= G.ROUND and cs - s * G.MARGIN <= G.ROUND
    grown = G.capacities([(c[0] + 1, c[1] + 1) for c in caps], G.REGROW)
    assert all(g[0] > c[0] and g[1] > c[1] for g, c in zip(grown, caps))
