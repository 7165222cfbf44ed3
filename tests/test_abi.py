"""C-ABI library checks that need no GPU: it builds, loads, exports every
entry point include/gbdbscan.h declares, and its host-only parts work."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "gbdbscan.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gd_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built_lib, gd):
    lib = gd.load_library()
    names = header_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name


def test_ctypes_signatures_cover_the_header(gd):
    from importlib import import_module
    api = import_module("fast-cuda-gpu-dbscan_gb300.api")
    assert sorted(n for n, _, _ in api.SIGNATURES) == header_functions()


def test_status_strings_and_version(built_lib, gd):
    lib = gd.load_library()
    assert lib.gd_abi_version() == 1
    assert lib.gd_status_string(0) == b"ok"
    assert lib.gd_status_string(4) == b"grid too large"


def test_import_dataset_csv_roundtrip(built_lib, gd, tmp_path, ds):
    pts = ds.blobs2d_100k(seed=3, scale=0.01).points
    path = tmp_path / "pts.csv"
    ds.write_csv(str(path), pts)
    got = gd.import_dataset(str(path), 2)
    assert np.array_equal(got, pts)
    got = gd.import_dataset(str(path), 2, max_points=10)
    assert np.array_equal(got, pts[:10])
    # the reference's own fixture format (test-datasets/ex.txt): "1,1" per line, CRLF tolerated
    p2 = tmp_path / "ex.txt"
    p2.write_bytes(b"1,1\r\n2,2\r\n3,3\r\n\r\n")
    assert gd.import_dataset(str(p2), 2).tolist() == [[1, 1], [2, 2], [3, 3]]


def test_import_dataset_binary(built_lib, gd, tmp_path):
    pts = np.random.default_rng(1).normal(size=(1000, 3))
    path = tmp_path / "pts.f64"
    pts.tofile(str(path))
    assert np.array_equal(gd.import_dataset(str(path), 3), pts)


def test_import_dataset_errors(built_lib, gd, tmp_path):
    with pytest.raises(gd.GdError) as e:
        gd.import_dataset(str(tmp_path / "missing.csv"), 2)
    assert e.value.status == 6
    bad = tmp_path / "bad.csv"
    bad.write_text("1,2\n3\n")
    with pytest.raises(gd.GdError) as e:
        gd.import_dataset(str(bad), 2)
    assert "line 2" in str(e.value)
    bad.write_text("1,x\n")
    with pytest.raises(gd.GdError):
        gd.import_dataset(str(bad), 2)
    with pytest.raises(gd.GdError) as e:
        gd.import_dataset(str(bad), 4)
    assert e.value.status == 1


def test_write_labels(built_lib, gd, tmp_path):
    lab = np.array([0, 0, -2, 1], dtype=np.int32)
    path = tmp_path / "out.txt"
    gd.write_labels(str(path), lab)
    assert path.read_text().split() == ["0", "0", "-2", "1"]


def test_context_without_gpu_reports_nodev(built_lib, gd):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gd.GdError) as e:
        gd.Context(0)
    assert e.value.status == 7


def test_server_argument_checks(built_lib, gd):
    import torch
    with pytest.raises(gd.GdError) as e:
        gd.Server(0, workers=0)
    assert e.value.status == 1
    with pytest.raises(gd.GdError) as e:
        gd.Server(0, hbm_budget_bytes=0)
    assert e.value.status == 1
    if torch.cuda.is_available():
        return
    with pytest.raises(gd.GdError) as e:
        gd.Server(0)
    assert e.value.status == 7


def test_cli_usage(built_lib):
    exe = os.path.join(os.path.dirname(built_lib), "gbdbscan_main")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2
    assert "Please provide the dataset file path" in r.stderr
