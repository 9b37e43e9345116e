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
