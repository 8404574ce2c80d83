"""Autotuner table: the tune-cache line format and the cache file (host
logic, no GPU), and on a GPU the measured table itself."""
import ctypes
import os

import numpy as np
import pytest

from spral_gb300 import _native


def _lib():
    return _native.lib()


def _ints(vals):
    a = np.asarray(vals, dtype=np.int32)
    return a, a.ctypes.data_as(ctypes.c_void_p)


def _format(key, table):
    a, p = _ints(table)
    buf = ctypes.create_string_buffer(512)
    n = _lib().spral_ssids_gpu_tune_format(key.encode(), p, len(a), buf, 512)
    return n, buf.value.decode()


def _parse(line):
    out = np.zeros(32, dtype=np.int32)
    key = ctypes.create_string_buffer(128)
    n = _lib().spral_ssids_gpu_tune_parse(line.encode(), key, 128,
                                          out.ctypes.data_as(ctypes.c_void_p), 32)
    return n, key.value.decode(), out[:max(n, 0)].tolist()


TABLE = [192, 5, 256, 128, 512, 128, 1024, 256, 2048, 256, 4096, 256]


def test_tune_line_round_trip():
    n, line = _format("NVIDIA_GB300-sm152-cc103", TABLE)
    assert n == len(line)
    assert line == ("spral_gb300-tune v1 NVIDIA_GB300-sm152-cc103 tc_min_cm=192 "
                    "bn=256:128,512:128,1024:256,2048:256,4096:256")
    m, key, vals = _parse(line)
    assert m == len(TABLE) and key == "NVIDIA_GB300-sm152-cc103" and vals == TABLE


@pytest.mark.parametrize("line", [
    "",
    "spral_gb300-tune v2 k tc_min_cm=192 bn=256:128",          # unknown version
    "other-tune v1 k tc_min_cm=192 bn=256:128",                 # wrong magic
    "spral_gb300-tune v1 k tc_min_cm=0 bn=256:128",             # crossover must be > 0
    "spral_gb300-tune v1 k tc_min_cm=192 bn=256:96",            # width the kernel lacks
    "spral_gb300-tune v1 k tc_min_cm=192 bn=512:128,256:128",   # classes not increasing
    "spral_gb300-tune v1 k tc_min_cm=192 bn=256:128,",          # trailing comma
    "spral_gb300-tune v1 k tc_min_cm=192 bn=",                  # no class
    "spral_gb300-tune v1 k tc_min_cm=192 bn=256:128 extra",     # trailing field
    "spral_gb300-tune v1 k tc_min_cm=19x bn=256:128",
])
def test_tune_line_rejects_malformed(line):
    assert _parse(line)[0] == -1


def test_tune_format_rejects_bad_tables():
    assert _format("k", [192, 1, 256, 96])[0] == -1          # bad width
    assert _format("k", [192, 2, 512, 128, 256, 128])[0] == -1  # not increasing
    assert _format("a key", TABLE)[0] == -1                  # key with a space
    assert _format("k", [192, 9] + [1, 64] * 9)[0] == -1     # too many classes


def test_tune_cache_store_and_lookup(tmp_path):
    path = str(tmp_path / "tune.txt")
    L = _lib()
    out = np.zeros(32, dtype=np.int32)
    op = out.ctypes.data_as(ctypes.c_void_p)
    # absent file: no entry
    assert L.spral_ssids_gpu_tune_cache_lookup(path.encode(), b"devA", op, 32) == 0
    a, p = _ints(TABLE)
    assert L.spral_ssids_gpu_tune_cache_store(path.encode(), b"devA", p, len(a)) == 0
    b_tab = [256, 1, 4096, 64]
    b_, bp = _ints(b_tab)
    assert L.spral_ssids_gpu_tune_cache_store(path.encode(), b"devB", bp, len(b_)) == 0
    assert L.spral_ssids_gpu_tune_cache_lookup(path.encode(), b"devA", op, 32) == len(TABLE)
    assert out[:len(TABLE)].tolist() == TABLE
    assert L.spral_ssids_gpu_tune_cache_lookup(path.encode(), b"devB", op, 32) == 4
    assert out[:4].tolist() == b_tab
    # replacing devA keeps devB; the file holds one line per device
    c_tab = [128, 1, 256, 256]
    c_, cp = _ints(c_tab)
    assert L.spral_ssids_gpu_tune_cache_store(path.encode(), b"devA", cp, len(c_)) == 0
    assert L.spral_ssids_gpu_tune_cache_lookup(path.encode(), b"devA", op, 32) == 4
    assert out[:4].tolist() == c_tab
    assert L.spral_ssids_gpu_tune_cache_lookup(path.encode(), b"devB", op, 32) == 4
    lines = open(path).read().splitlines()
    assert len(lines) == 2 and all(l.startswith("spral_gb300-tune v1 ") for l in lines)
    assert not [f for f in os.listdir(tmp_path) if ".tmp" in f]
    # too little room for the table
    assert L.spral_ssids_gpu_tune_cache_lookup(path.encode(), b"devB", op, 3) == -1


def test_tune_cache_skips_malformed_lines(tmp_path):
    path = tmp_path / "tune.txt"
    good = "spral_gb300-tune v1 devA tc_min_cm=192 bn=256:128,4096:256"
    path.write_text("garbage line\n" + good + "\nspral_gb300-tune v1 devA tc_min_cm=-3 bn=1:64\n")
    out = np.zeros(32, dtype=np.int32)
    n = _lib().spral_ssids_gpu_tune_cache_lookup(str(path).encode(), b"devA",
                                                 out.ctypes.data_as(ctypes.c_void_p), 32)
    assert n == 6 and out[:6].tolist() == [192, 2, 256, 128, 4096, 256]


@pytest.mark.gpu
def test_tune_table_is_measured_and_cached(tmp_path, monkeypatch):
    L = _lib()
    out = np.zeros(32, dtype=np.int32)
    op = out.ctypes.data_as(ctypes.c_void_p)
    n = L.spral_ssids_gpu_tune_table(op, 32)
    assert n >= 4
    tab = out[:n].tolist()
    assert tab[0] == L.spral_ssids_gpu_tc_crossover()
    nb = tab[1]
    ms = tab[2::2][:nb]
    assert ms == sorted(ms) and all(w in (64, 128, 256) for w in tab[3::2][:nb])
    key = ctypes.create_string_buffer(256)
    assert L.spral_ssids_gpu_tune_device_key(key, 256) > 0
    assert " " not in key.value.decode()
    # the table round-trips through the cache format
    a, p = _ints(tab)
    path = str(tmp_path / "t.txt")
    assert L.spral_ssids_gpu_tune_cache_store(path.encode(), key.value, p, len(a)) == 0
    assert L.spral_ssids_gpu_tune_cache_lookup(path.encode(), key.value, op, 32) == n
    assert out[:n].tolist() == tab
