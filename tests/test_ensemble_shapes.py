"""Host logic of the batch's tile shapes (no GPU): tile counts as fd_batch
builds them and the strip heights that fill whole rounds of the persistent
grid, which the autotuner adds to its candidates."""
from fingering_dynamics_gb300.ensemble import ensemble_specs, round_filling_rows, tile_count


def test_tile_count_by_hand():
    sizes = [(128, 512), (256, 2048), (100, 300)]
    # 512/128 = 4 bands x 2 strips; 16 bands x 4 strips; 3 bands x 2 strips (100 = 64 + 36)
    assert tile_count(sizes, 128, 64) == 4 * 2 + 16 * 4 + 3 * 2
    # strips taller than a lattice are one strip
    assert tile_count(sizes, 128, 1000) == 4 + 16 + 3
    assert tile_count([(7, 64)], 64, 16) == 1


def test_round_filling_rows_fit_their_rounds():
    specs = ensemble_specs(96, seed=2024)
    sizes = [(s.H, s.W) for s in specs]
    grid = 760
    rows = round_filling_rows(sizes, 128, grid, max_rounds=8, min_fill=0.9)
    assert rows, "no strip height fills whole rounds"
    for h in rows:
        t = tile_count(sizes, 128, h)
        r = -(-t // grid)
        assert t <= r * grid and t >= 0.9 * r * grid
        # the next shorter strip needs more tiles than the rounds hold
        if h > 16:
            assert tile_count(sizes, 128, h - 1) > r * grid
    # the 128 x 64 shape of this ensemble (3,500 tiles = 4.6 rounds) is not among them
    assert 64 not in rows or tile_count(sizes, 128, 64) >= 0.9 * 5 * grid
