"""Host-side arithmetic of the benchmark: the whole-job metric and the
roofline of the dominant kernel, from a synthetic per-kernel profile (no GPU
needed)."""
import math

import bench


def test_job_value_is_whole_job_throughput():
    # 2 replicas x 6,291,456 prisms x 5 steps in 2 s -> 31.5 Mcell-steps/s
    assert math.isclose(bench.job_value(2, 6291456, 5, 2000.0), 2 * 6291456 * 5 / 2.0 / 1e6)


def test_roofline_of_the_mixed_solver():
    prisms, iters = 6291456, 1000
    # k_in_pv: 1000 busy launches plus idle slots, 67 ms in total
    prof = {"k_in_pv": (1100, 67.0), "k_in_st": (1100, 40.0), "k_mix_update": (30, 4.0), "k_stage_rhs": (3, 7.0)}
    roof, shares, total = bench.roofline(prof, iters, prisms, mixed=True)
    peak, kind = bench.load_peaks()
    assert roof["kernel"] == "k_in_pv" and roof["bound"] == "hbm" and roof["unit"] == "GB/s"
    # algorithmic bytes: 11 FP32 words a prism, counted per busy iteration
    bpl = 11 * 4 * prisms
    assert roof["algorithmic_bytes_per_launch"] == bpl
    achieved = bpl * iters / 0.067 / 1e9
    assert math.isclose(roof["achieved"], round(achieved, 1))
    assert math.isclose(roof["frac"], round(achieved / peak, 4))
    assert roof["peak"] == peak and roof["peak_kind"] == kind
    assert math.isclose(roof["avg_launch_ms"], 67.0 / iters)
    assert math.isclose(total, 118.0)
    assert math.isclose(sum(shares.values()), 1.0, abs_tol=1e-3)
    assert roof["fp64_tflops"] is None  # FP32 kernel


def test_kernel_times_are_per_launch_that_did_work():
    # iteration passes per iteration, hand-over kernels per FP64 update,
    # everything else per launch; kernels that never launched are left out
    prof = {"k_in_pv": (1100, 67.0), "k_in_st": (1100, 40.0), "k_mix_scale": (140, 3.0),
            "k_stage_rhs": (3, 7.2), "k_project": (0, 0.0)}
    us = bench.kernel_us(prof, iters=1000, updates=30)
    assert us == {"k_in_pv": 67.0, "k_in_st": 40.0, "k_mix_scale": 100.0, "k_stage_rhs": 2400.0}


def test_roofline_of_the_fp64_solver_reports_its_fp64_rate():
    prisms, iters = 1048576, 500
    prof = {"k_bicg_x": (500, 17.5), "k_bicg_p": (500, 5.0)}
    roof, _, _ = bench.roofline(prof, iters, prisms, mixed=False)
    assert roof["kernel"] == "k_bicg_x"
    assert roof["algorithmic_bytes_per_launch"] == 8 * 8 * prisms
    flops = bench.FLOPS["stored"]["k_bicg_x"] * prisms * iters
    assert math.isclose(roof["fp64_tflops"], round(flops / 0.0175 / 1e12, 3))


def test_fp64_spmv_flops_follow_the_form_that_runs():
    # the stored-coupling SpMV executes five FMAs a row plus its dots; the
    # matrix-free one two more multiplies a coupling (ten a row)
    prisms, iters = 1048576, 500
    prof = {"k_bicg_spmv_t": (500, 20.0)}
    st, _, _ = bench.roofline(prof, iters, prisms, mixed=False, spmv="stored")
    mf, _, _ = bench.roofline(prof, iters, prisms, mixed=False, spmv="matrix-free")
    assert bench.FLOPS["stored"]["k_bicg_spmv_t"] == 5 * 2 + 2 * 2
    assert bench.FLOPS["matrix-free"]["k_bicg_spmv_t"] - bench.FLOPS["stored"]["k_bicg_spmv_t"] == 10
    assert math.isclose(st["fp64_tflops"], round(14 * prisms * iters / 0.020 / 1e12, 3))
    assert math.isclose(mf["fp64_tflops"], round(24 * prisms * iters / 0.020 / 1e12, 3))


def test_step_bytes_count_iterations_updates_and_stage_kernels():
    prisms = 1000
    prof = {"k_in_pv": (1100, 67.0), "k_in_st": (1100, 40.0), "k_mix_update": (300, 4.0),
            "k_mix_scale": (300, 2.0), "k_stage_rhs": (6, 7.0), "k_project": (6, 3.0), "other": (4, 0.1),
            "k_bicg_p": (0, 0.0)}
    bstep, b_it, b_up, b_fix = bench.step_bytes(prof, iters=1000, updates=40, steps=2, prisms=prisms, mixed=True)
    w = bench.WORDS_MIXED
    assert b_it == (w["k_in_pv"] + w["k_in_st"]) * 8 * prisms
    assert b_up == (w["k_mix_update"] + w["k_mix_scale"]) * 8 * prisms
    assert b_fix == (bench.WORDS["k_stage_rhs"] * 6 + bench.WORDS["k_project"] * 6 + 3 * 4) * 8 * prisms / 2
    assert math.isclose(bstep, b_fix + (b_it * 1000 + b_up * 40) / 2)


def test_fp64_roofline_takes_the_lower_roof():
    prisms, iters = 1048576, 500
    prof = {"k_bicg_x": (500, 17.5)}
    roof, _, _ = bench.roofline(prof, iters, prisms, mixed=False, fp64_peak=1.2)
    assert roof["fp64_peak_tflops"] == 1.2
    assert math.isclose(roof["fp64_frac"], round(roof["fp64_tflops"] / 1.2, 4))
    assert roof["bound"] == ("fp64" if roof["fp64_frac"] > roof["frac"] else "hbm")
