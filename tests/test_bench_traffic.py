"""The bench line's roofline `traffic` comes from a committed per-kernel capture
(profiles/traffic_<workload>_<precision>.json) only when that capture was taken
on the sources being measured and on the same point count; otherwise it is null
and the line says why.  CPU only: the captures' metadata and bench.py's check."""
import importlib
import importlib.util
import json
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _digest():
    return importlib.import_module("fast-cuda-gpu-dbscan_gb300.build").source_digest()


def test_committed_captures_describe_the_full_workloads():
    for name, points in (("traffic_zipf2d_10m_fp64.json", 10_000_000),
                         ("traffic_aniso3d_20m_fp32band.json", 20_000_000)):
        with open(os.path.join(ROOT, "profiles", name)) as f:
            tj = json.load(f)
        assert tj["points"] == points
        assert tj["captured_points"] < points and tj["scale_to_full"] * tj["captured_points"] == points
        assert set(tj["phases"]) == {"ms_index", "ms_core", "ms_union", "ms_label"}
        # the step total is the sum of its phases and of its kernels
        assert abs(sum(tj["phases"].values()) - tj["dram_bytes_per_step"]) < 1.0
        kern = sum(k["dram_bytes"] for k in tj["kernels"].values())
        assert abs(kern - tj["dram_bytes_per_step"]) <= 1e-6 * tj["dram_bytes_per_step"] + 1.0
        assert len(tj["source_digest"]) == 16


def test_traffic_used_only_for_matching_sources_and_size(tmp_path, monkeypatch):
    b = _bench()
    prof = tmp_path / "profiles"
    prof.mkdir()
    src = os.path.join(ROOT, "profiles", "traffic_zipf2d_10m_fp64.json")
    with open(src) as f:
        tj = json.load(f)
    monkeypatch.setattr(b, "ROOT", str(tmp_path))
    # matching sources and size: used, and the line names the file and sources
    tj["source_digest"] = _digest()
    (prof / "traffic_zipf2d_10m_fp64.json").write_text(json.dumps(tj))
    got, why = b.recorded_traffic("zipf2d_10m", "fp64", 10_000_000)
    assert got is not None and got["dram_bytes_per_step"] == tj["dram_bytes_per_step"]
    assert "traffic_zipf2d_10m_fp64.json" in why and _digest() in why
    # another point count (a --scale run): not used
    got, why = b.recorded_traffic("zipf2d_10m", "fp64", 2_000_000)
    assert got is None and "points" in why
    # other sources: not used
    tj["source_digest"] = "0" * 16
    (prof / "traffic_zipf2d_10m_fp64.json").write_text(json.dumps(tj))
    got, why = b.recorded_traffic("zipf2d_10m", "fp64", 10_000_000)
    assert got is None and "other sources" in why
    # no capture at all
    got, why = b.recorded_traffic("aniso3d_20m", "fp32band", 20_000_000)
    assert got is None
