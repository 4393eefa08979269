"""The roofline numerator of bench.py (algorithmic bytes per launch) on the 3D dambreak's
list figures: the per-array accounting its docstring states, for the fused FP32-mixed
step forms and the unfused stage sequence."""
import bench

N_TOTAL, N_FLUID = 2_324_868, 911_754
LISTS = {"entries_real": 110_158_889, "entries_dummy": 2_574_071, "listed_dummies": 115_380}


def test_rates_bytes_leapfrog_cspm():
    n_vis = N_FLUID + LISTS["listed_dummies"]
    want = n_vis * 32 + N_FLUID * (16 + 4 + 4 + 26 + 20) + 4 * LISTS["entries_real"]
    assert bench.algorithmic_bytes("rates", N_TOTAL, N_FLUID, "fp32_mixed", True, LISTS, "lf") == want


def test_fused_forms_differ_by_the_cspm_factor_bytes():
    def rates(corr, fused):
        return bench.algorithmic_bytes("rates", N_TOTAL, N_FLUID, "fp32_mixed", corr, LISTS, fused)
    assert rates(True, "lf") - rates(True, None) == 2 * N_FLUID
    assert rates(False, "lf") - rates(False, None) == 2 * N_FLUID
    assert rates(True, "se") - rates(True, None) == 4 * N_FLUID
    assert rates(False, "se") - rates(False, None) == 4 * N_FLUID


def test_correction_bytes_fused_visit_flow_only():
    fused = bench.algorithmic_bytes("kernel_corr", N_TOTAL, N_FLUID, "fp32_mixed", True, LISTS, "se")
    assert fused == N_FLUID * (36 + 4 + 24) + 4 * LISTS["entries_real"]
    alone = bench.algorithmic_bytes("kernel_corr", N_TOTAL, N_FLUID, "fp32_mixed", True, LISTS)
    assert alone > fused


def test_boundary_bytes_unchanged_by_fusion():
    a = bench.algorithmic_bytes("boundary", N_TOTAL, N_FLUID, "fp32_mixed", True, LISTS, "lf")
    b = bench.algorithmic_bytes("boundary", N_TOTAL, N_FLUID, "fp32_mixed", True, LISTS)
    assert a == b == 57_381_404


def test_traffic_read_from_the_committed_capture():
    """roofline.traffic: the rates capture's DRAM bytes per launch (profiles/), scaled by the
    list entries of the run against those of the capture."""
    traffic, src = bench.read_profile_traffic("rates_fp32_mixed_3d_dambreak", LISTS["entries_real"])
    assert src["profile"] == "profiles/rates_fp32_mixed_3d_dambreak.md"
    assert src["capture_list_entries"] > 0 and src["capture_dram_bytes_per_launch"] > 0
    want = src["capture_dram_bytes_per_launch"] * LISTS["entries_real"] / src["capture_list_entries"]
    assert abs(traffic - want) <= 1e-6 * want
    # the measured traffic is within a few percent of the algorithmic bytes of the same launch
    alg = bench.algorithmic_bytes("rates", N_TOTAL, N_FLUID, "fp32_mixed", True, LISTS, "lf")
    assert 0.95 < traffic / alg < 1.10
    missing, why = bench.read_profile_traffic("no_such_kernel", LISTS["entries_real"])
    assert missing is None and "missing" in why
