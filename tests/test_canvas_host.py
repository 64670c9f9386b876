"""Host-side layout of the uneven multi-instance iteration (no GPU):
canvas_layout places every instance's grid on one canvas, split_by_work
divides the instances between canvases."""
import numpy as np

from ernn_gb300 import harness as Hn
from ernn_gb300 import configs as Cf


def _rects(ws, x0, y0):
    return [(x0[k], y0[k], x0[k] + w.nx, y0[k] + w.ny) for k, w in enumerate(ws)]


def test_canvas_layout_regions_are_apart_and_aligned():
    ws = Cf.multi_instances(64)
    X, Y, x0, y0 = Hn.canvas_layout(ws)
    assert Y % 64 == 0
    r = _rects(ws, x0, y0)
    for k, (a0, b0, a1, b1) in enumerate(r):
        assert 0 <= a0 and a1 <= X and 0 <= b0 and b1 <= Y
        assert b0 % 32 == 0  # rows of every region start on 128-byte lines
        for (c0, d0, c1, d1) in r[k + 1:]:
            # at least one row or four columns between any two regions: the
            # cells between them are the instances' zero ghost rings
            apart_rows = a1 + 1 <= c0 or c1 + 1 <= a0
            apart_cols = b1 + 4 <= d0 or d1 + 4 <= b0
            assert apart_rows or apart_cols
    # the packing wastes less than a fifth of the canvas
    assert sum(w.nx * w.ny for w in ws) >= 0.8 * X * Y


def test_canvas_layout_column_alignment_option():
    ws = Cf.multi_instances(8, sides=[128, 192, 256, 128, 320, 128, 192, 256])
    _, _, _, y0 = Hn.canvas_layout(ws, col_align=4)
    assert all(v % 4 == 0 for v in y0)
    _, _, _, y0 = Hn.canvas_layout(ws)
    assert all(v % 32 == 0 for v in y0)


def test_split_by_work_balances_and_covers():
    ws = Cf.multi_instances(64)
    work = np.array([w.nx * w.ny * w.nt for w in ws], dtype=np.float64)
    for parts in (1, 2, 3, 4):
        m = Hn.split_by_work(ws, parts)
        assert sorted(k for g in m for k in g) == list(range(len(ws)))
        assert all(g == sorted(g) for g in m)
        loads = [work[g].sum() for g in m]
        # greedy largest-first: within the largest single instance of equal
        assert max(loads) - min(loads) <= work.max()
    assert Hn.split_by_work(ws, 2) == Hn.split_by_work(ws, 2)  # deterministic
    # fewer instances than parts: empty parts are dropped
    assert len(Hn.split_by_work(ws[:2], 4)) == 2


def test_canvas_layout_random_instance_sets():
    """Seeded random sets of 1-40 instances (heights 4-300, widths multiples
    of 4 up to 300): every placement satisfies what the library checks for
    ERNN_FLAG_INSTANCES (inside the canvas, canvas width and first columns
    multiples of 4, any two regions at least one row or one column apart)
    plus the layout's own alignment and gap."""
    from types import SimpleNamespace
    rng = np.random.default_rng(7)
    for _ in range(200):
        n = int(rng.integers(1, 41))
        ws = [SimpleNamespace(nx=int(rng.integers(4, 301)), ny=4 * int(rng.integers(1, 76))) for _ in range(n)]
        for align in (32, 4):
            X, Y, x0, y0 = Hn.canvas_layout(ws, col_align=align)
            # the canvas width: a multiple of the alignment (so of 4, as the
            # tiled kernels need), below the 16-bit limit of the tile table
            assert Y % align == 0 and Y % 4 == 0 and X <= 65535 and Y <= 65535
            r = _rects(ws, x0, y0)
            for k, (a0, b0, a1, b1) in enumerate(r):
                assert 0 <= a0 and a1 <= X and 0 <= b0 and b1 <= Y
                assert b0 % align == 0
                for (c0, d0, c1, d1) in r[k + 1:]:
                    assert a1 + 1 <= c0 or c1 + 1 <= a0 or b1 + 4 <= d0 or d1 + 4 <= b0
