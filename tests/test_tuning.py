"""Launch-parameter table (ibim_tuning_*) without a GPU: rows by order and size, file loading,
rejected values."""

import os
import tempfile

import pytest

import ibim


@pytest.fixture
def clean_table():
    lib = ibim.lib()
    lib.ibim_tuning_clear()
    yield lib
    lib.ibim_tuning_clear()
    if os.path.exists(ibim.TUNING_TABLE):
        lib.ibim_tuning_load(ibim.TUNING_TABLE.encode())


def test_defaults_without_rows(clean_table):
    assert ibim.tuning_get(5, 400_000) == dict(near_seg_pairs=1 << 17, nearff_seg_pairs=1 << 14, tc_form=2)


def test_row_with_largest_min_points_applies(clean_table):
    lib = clean_table
    assert lib.ibim_tuning_set(5, 0, 1 << 16, 1 << 13, 2) == ibim.OK
    assert lib.ibim_tuning_set(5, 100_000, 1 << 18, 1 << 15, 4) == ibim.OK
    assert ibim.tuning_get(5, 50_000) == dict(near_seg_pairs=1 << 16, nearff_seg_pairs=1 << 13, tc_form=2)
    assert ibim.tuning_get(5, 100_000) == dict(near_seg_pairs=1 << 18, nearff_seg_pairs=1 << 15, tc_form=4)
    assert ibim.tuning_get(4, 100_000)["near_seg_pairs"] == 1 << 17  # other orders keep the defaults
    assert lib.ibim_tuning_set(5, 100_000, 1 << 15, 1 << 14, 2) == ibim.OK  # replaces the row
    assert ibim.tuning_get(5, 10 ** 7)["near_seg_pairs"] == 1 << 15


def test_load_table_file(clean_table):
    lib = clean_table
    with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
        f.write("# comment\n5 0 65536 8192 2   # note\n\n6 1000 262144 32768 4\n")
        path = f.name
    try:
        assert lib.ibim_tuning_load(path.encode()) == ibim.OK
        assert ibim.tuning_get(6, 5000) == dict(near_seg_pairs=262144, nearff_seg_pairs=32768, tc_form=4)
        assert ibim.tuning_get(5, 5000)["near_seg_pairs"] == 65536
    finally:
        os.unlink(path)


def test_rejects_bad_rows(clean_table):
    lib = clean_table
    assert lib.ibim_tuning_set(5, 0, 10, 1 << 14, 2) == ibim.ERR_INVALID_ARGUMENT
    assert lib.ibim_tuning_set(5, 0, 1 << 17, 1 << 14, 3) == ibim.ERR_INVALID_ARGUMENT
    assert lib.ibim_tuning_set(1, 0, 1 << 17, 1 << 14, 2) == ibim.ERR_INVALID_ARGUMENT
    with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
        f.write("5 0 131072\n")
        path = f.name
    try:
        assert lib.ibim_tuning_load(path.encode()) == ibim.ERR_IO
    finally:
        os.unlink(path)
    assert lib.ibim_tuning_load(b"/nonexistent/table.txt") == ibim.ERR_IO


def test_committed_table_parses():
    if not os.path.exists(ibim.TUNING_TABLE):
        pytest.skip("no table measured yet")
    rows = [ln.split("#")[0].split() for ln in open(ibim.TUNING_TABLE)]
    rows = [r for r in rows if r]
    assert rows and all(len(r) == 5 for r in rows)
    assert ibim.lib().ibim_tuning_load(ibim.TUNING_TABLE.encode()) == ibim.OK
