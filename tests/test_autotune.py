"""The autotuner's host logic: bucketing (must agree with the library's), table fill and format."""
from __future__ import annotations

from sdfb import autotune


def test_buckets_match_library_rule():
    assert [autotune.bucket_tris(t) for t in (1, 2, 3, 1280, 81920, 327680, 1 << 40)] == [0, 1, 1, 10, 16, 18, 31]
    assert [autotune.bucket_grid(n) for n in (1, 16, 31, 64, 128, 256, 511, 512, 1 << 14)] == [0, 0, 0, 2, 3, 4, 4, 5, 7]


def test_fill_table_nearest(tmp_path):
    measured = {(10, 2): (2, 1, 32, -1), (16, 4): (4, 3, 64, 1024)}
    table = autotune.fill_table(measured)
    assert len(table) == 32 * 8
    assert table[(10, 2)] == (2, 1, 32, -1) and table[(16, 4)] == (4, 3, 64, 1024)
    assert table[(0, 0)] == (2, 1, 32, -1) and table[(31, 7)] == (4, 3, 64, 1024)
    path = tmp_path / "t.tsv"
    autotune.write_table(str(path), table, measured, {(10, 2): 1.0, (16, 4): 2.0}, ["test"])
    rows = [l.split("#")[0].split() for l in path.read_text().splitlines() if not l.startswith("#")]
    assert len(rows) == 256
    row = [r for r in rows if r[:2] == ["16", "4"]][0]
    assert row == ["16", "4", "4", "2", "64", "1024"]  # tile written 0-based
    assert [r for r in rows if r[:2] == ["10", "2"]][0][5] == "0"  # never defer


def test_batch_line_written_and_replaced(tmp_path):
    path = str(tmp_path / "t.tsv")
    table = autotune.fill_table({(16, 4): (4, 3, 64, 1024)})
    autotune.write_table(path, table, {(16, 4): (4, 3, 64, 1024)}, {(16, 4): 2.0}, ["test"])
    autotune.write_batch_line(path, (5, 32, -1), "faster")
    autotune.write_batch_line(path, (6, 64, 512), "faster again")
    lines = open(path).read().splitlines()
    batch = [l for l in lines if l.startswith("batch ")]
    assert batch == ["batch 5 64 512  # faster again"]  # tile 0-based, one line only
    assert len([l for l in lines if l and not l.startswith("#") and not l.startswith("batch")]) == 256
    autotune.write_batch_line(path, None, "kept")
    lines = open(path).read().splitlines()
    assert not [l for l in lines if l.startswith("batch ")] and lines[-1] == "# batch: kept"


def test_tune_batch_descends_and_keeps_the_table_when_nothing_is_faster():
    # a fake timer: the table's choice (None) takes 100 ms; tile 5 saves 5 ms, stack 32 saves 10
    def fake(p):
        if p is None:
            return 100.0
        tile, stack, budget = p
        return 105.0 - 5.0 * (tile == 5) - 10.0 * (stack == 32)
    best, best_ms, table_ms = autotune.tune_batch(fake, log=lambda *a: None)
    assert best[:2] == (5, 32) and best_ms == 90.0 and table_ms == 100.0
    best, best_ms, table_ms = autotune.tune_batch(lambda p: 100.0 if p is None else 120.0, log=lambda *a: None)
    assert best is None and best_ms == table_ms == 100.0
