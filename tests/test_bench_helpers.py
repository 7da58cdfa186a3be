"""The benchmark's host-side arithmetic (no GPU): the per-layer roofline bound
of the denoiser, the whole-job rate of a weak-scaling run, the per-launch
traversal roofline against HBM and L2, and the profile constants and CPU
calibration the benchmark line reads."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _layer(ci, co, level=0, c1=None, up1=0):
    return {"cin_pad": ci, "cout_pad": co, "c1_pad": ci if c1 is None else c1, "up1": up1, "level": level}


def test_layer_bound_takes_the_larger_of_tensor_and_memory_time():
    px = 1 << 20
    tflops, gbs = 1000.0, 5000.0
    # 16 -> 16 channels: 2 * 9 * 256 = 4,608 FLOP and (16 + 16) * 2 = 64 B per
    # pixel: memory-bound (64 B / 5 TB/s > 4.6 kFLOP / 1 PFLOP/s)
    L = _layer(16, 16)
    want = 64 * px / (gbs * 1e9) * 1e3
    assert abs(bench.layer_bound_ms([L], px, tflops, gbs, train=False) - want) < 1e-12
    # 256 -> 256 channels: tensor-bound
    L = _layer(256, 256)
    want = 2 * 9 * 256 * 256 * px / (tflops * 1e12) * 1e3
    assert abs(bench.layer_bound_ms([L], px, tflops, gbs, train=False) - want) < 1e-12


def test_layer_bound_training_adds_two_gradient_passes_and_scales_by_level():
    px = 1 << 20
    L0 = _layer(256, 256, level=0)
    L1 = _layer(256, 256, level=1)
    fwd = bench.layer_bound_ms([L0], px, 1000.0, 5000.0, train=False)
    assert abs(bench.layer_bound_ms([L0], px, 1000.0, 5000.0, train=True) - 3 * fwd) < 1e-12
    # a level-1 layer sees a quarter of the pixels
    assert abs(bench.layer_bound_ms([L1], px, 1000.0, 5000.0, train=False) - fwd / 4) < 1e-12


def test_upsampled_source_counts_a_quarter_of_its_bytes():
    px = 1 << 20
    # 64 upsampled channels + 32 skip channels -> 32, memory-bound
    L = _layer(96, 32, c1=64, up1=1)
    want = ((64 / 4 + 32) + 32) * 2 * px / 1e9 * 1e3
    got = bench.layer_bound_ms([L], px, 1e9, 1.0, train=False)  # 1 GB/s: memory-bound
    assert abs(got - want) < 1e-9 * want


def test_job_rate_is_weak_scaling_over_the_slowest_rank():
    assert bench.job_rate(100, 2.0, 1) == 50.0
    assert bench.job_rate(100, 2.0, 4) == 200.0
    assert bench.reduce_max(3.5, 1) == 3.5


def test_traversal_roofline_per_launch_against_hbm_and_l2():
    l2 = {"peak_gbs": 20000.0}
    r = bench.traversal_roofline(bytes_frame=22e9, launches_frame=11, ms_frame=33.0, hbm=6800.0,
                                 hbm_kind="measured", l2=l2)
    # 2 GB per launch in 3 ms: 666.7 GB/s
    assert abs(r["bytes_per_launch"] - 2e9) < 1e-3 and abs(r["avg_launch_ms"] - 3.0) < 1e-12
    assert abs(r["achieved"] - 2e9 / 3e-3 / 1e9) < 1e-9
    assert abs(r["frac"] - r["achieved"] / 6800.0) < 1e-12
    assert abs(r["l2"]["frac"] - r["achieved"] / 20000.0) < 1e-12
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"


def test_profile_facts_reads_key_value_lines(tmp_path, monkeypatch):
    prof = tmp_path / "profiles"
    prof.mkdir()
    (prof / "x.txt").write_text("# a comment 1.0\nwarp_inst_per_sample 356.2\nnot_a_number abc\n\nfoo 2e3 trailing\n")
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.profile_facts("x.txt") == {"warp_inst_per_sample": 356.2, "foo": 2000.0}
    assert bench.profile_facts("missing.txt") == {}


def test_committed_profile_constants_are_readable():
    """The constants the bench combines with its own timings exist."""
    f = bench.profile_facts("k_shade_issue.txt")
    assert f["warp_inst_per_sample"] > 0 and f["fp32_ops_per_sample"] > 0
    c = bench.profile_facts("cornell_c1_issue.txt")
    assert c["thread_inst_per_frame"] > c["warp_inst_per_frame"] > 0
    assert bench.profile_facts("k_extend_traffic.txt")["dram_bytes_per_extension_ray"] > 0


def test_cpu_calibration_reports_the_three_ratios():
    c = bench.cpu_calibration()
    assert c is not None
    assert set(c["restatement_over_reference_speed"]) == {"paths_d12", "paths_d5", "render_d5"}
    assert all(v > 0 for v in c["restatement_over_reference_speed"].values())
