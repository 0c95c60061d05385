"""The benchmark's DRAM-traffic record: parsed from an ncu CSV capture of the
transport launches, keyed to the hash of the kernel's sources, and reported
only while that hash matches the kernel the benchmark runs."""
import json

import pytest

import bench

_HEAD = ('"ID","Process ID","Process Name","Host Name","Kernel Name","Context","Stream","Block Size",'
         '"Grid Size","Device","CC","Section Name","Metric Name","Metric Unit","Metric Value"\n')


def _row(i, kernel, metric, unit, value):
    return (f'"{i}","1","python3.12","127.0.0.1","{kernel}","1","13","(256, 1, 1)","(760, 1, 1)","0","10.3",'
            f'"Command line profiler metrics","{metric}","{unit}","{value}"\n')


def _capture(tmp_path):
    k = "void mcfl_transport_fast<1, 0, 0, 256, 5, 0, 0, 0>(McflLaunch)"
    text = "==PROF== Connected to process 1\n" + _HEAD
    text += _row(0, k, "dram__bytes_read.sum", "Mbyte", "36.37")
    text += _row(0, k, "dram__bytes_write.sum", "byte", "512")
    text += _row(0, k, "gpu__time_duration.sum", "ms", "415.07")
    text += _row(1, "void other_kernel(int)", "dram__bytes_read.sum", "Gbyte", "9.0")
    text += _row(2, k, "dram__bytes_read.sum", "byte", "6,969,856")
    text += _row(2, k, "dram__bytes_write.sum", "byte", "0")
    text += _row(2, k, "gpu__time_duration.sum", "ns", "658393120")
    p = tmp_path / "traffic.csv"
    p.write_text(text)
    return str(p)


def test_record_from_capture_and_build_identity(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "TRAFFIC_FILE", str(tmp_path / "record.json"))
    rec = bench.traffic_from_csv(_capture(tmp_path), "the capture command")
    assert [x["launch"] for x in rec["launches"]] == [0, 1]  # the other kernel is left out
    assert rec["launches"][0]["dram_bytes"] == pytest.approx(36.37e6 + 512)
    assert rec["launches"][0]["duration_s"] == pytest.approx(0.41507)
    assert rec["launches"][1]["dram_bytes"] == pytest.approx(6969856.0)
    assert rec["launches"][1]["duration_s"] == pytest.approx(0.65839312)
    assert rec["dram_bytes_per_launch"] == pytest.approx((36.37e6 + 512 + 6969856.0) / 2)
    assert rec["source_sha256"] == bench.kernel_source_sha()
    value, note = bench.traffic_of_this_build()
    assert value == pytest.approx(rec["dram_bytes_per_launch"]) and "the capture command" in note
    # a record of another build of the kernel is not reported
    rec["source_sha256"] = "0" * 64
    (tmp_path / "record.json").write_text(json.dumps(rec))
    value, note = bench.traffic_of_this_build()
    assert value is None and "another build" in note


def test_no_record(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "TRAFFIC_FILE", str(tmp_path / "missing.json"))
    value, note = bench.traffic_of_this_build()
    assert value is None and "no ncu capture" in note
