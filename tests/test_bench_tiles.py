"""bench.py's mapping of the batch autotuner's report to each grid's flux tile
(the tile of the grid's size class), as gfm_batch_autotune assigns them."""
import os
import sys
from types import SimpleNamespace

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def grid(nx, ny, g=2):
    return SimpleNamespace(Nx=nx, Ny=ny, numGC=g)


def test_each_grid_takes_its_size_class_tile():
    report = {"classes": [{"max_padded_cells": 131072, "tile": "32x8"},
                          {"max_padded_cells": 524288, "tile": "16x16"},
                          {"max_padded_cells": -1, "tile": "16x32"}], "tiles": "per class"}
    descs = [grid(96, 48), grid(508, 252), grid(512, 252), grid(1000, 400)]
    # padded cells: 100*52 = 5200; 512*256 = 131072 (not below the first bound);
    # 516*256 = 132096; 1004*404 = 405616 (below 2^19)
    assert bench.tiles_from_report(report, descs) == ["32x8", "16x16", "16x16", "16x16"]
    descs = [grid(1000, 600)]   # 1004*604 = 606416: the unbounded class
    assert bench.tiles_from_report(report, descs) == ["16x32"]


def test_classes_without_instances_are_absent_from_the_report():
    report = {"classes": [{"max_padded_cells": -1, "tile": "16x16"}], "tiles": "per class"}
    assert bench.tiles_from_report(report, [grid(64, 64), grid(900, 900)]) == ["16x16", "16x16"]
    report = {"classes": [{"max_padded_cells": 131072, "tile": "32x8"}]}
    assert bench.tiles_from_report(report, [grid(900, 900)]) == [None]
