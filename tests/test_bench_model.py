"""bench.py's minimum-traffic byte model and the figures it reads from the
committed ncu summaries, on the CPU.

  - the CG iteration model (40 B + 148 N) and the step kernels' models at
    the sizes of the 40 nm and 61.25 nm spheres, against the per-launch
    byte counts the bench lines report;
  - the ncu summaries parse, and the memory-resident one's per-iteration
    DRAM figure is its per-launch figure over the run's iterations.
"""
import pytest

import bench

# corner nodes, elements, edges of the synthetic spheres (ffea_gb300.workloads)
SPHERE40 = (146_737, 823_968, 989_154)
SPHERE61 = (514_965, 2_958_132, 3_516_752)


def test_cg_iteration_bytes():
    assert bench.cg_iteration_bytes(SPHERE40[0], SPHERE40[2]) == 106_718_876
    assert bench.cg_iteration_bytes(SPHERE61[0], SPHERE61[2]) == 378_153_580
    # one more edge adds two 3x3 blocks (36 B values + 4 B column each)
    assert bench.cg_iteration_bytes(10, 11) - bench.cg_iteration_bytes(10, 10) == 80


def test_step_kernel_bytes():
    N, E, ed = SPHERE40
    got = bench.step_kernel_bytes(N, E, ed, 1_135_891)
    assert got == {"noise": 24_831_948, "elements": 140_187_468, "assemble": 162_194_292, "nodes": 55_081_744}


def test_ncu_summaries_parse():
    per_launch40 = bench.ncu_traffic("k_cg", "sphere40")
    assert per_launch40 is not None and per_launch40 > 0
    per_launch61 = bench.ncu_traffic("k_cg", "sphere61")
    per_it61 = bench.ncu_summary_value("dram_bytes_per_iteration", workload="sphere61")
    assert per_launch61 is not None and per_it61 is not None
    # 86.33 iterations a step in the captured run
    assert per_it61 == pytest.approx(per_launch61 / 86.33, rel=2e-3)
    # DRAM bytes of the memory-resident solve stay within 25 % of the model
    model = bench.cg_iteration_bytes(SPHERE61[0], SPHERE61[2])
    assert 0.75 * model < per_it61 < 1.25 * model
    assert bench.ncu_summary_value("no_such_key") is None


def test_measured_peak():
    peak, source = bench.measured_peak()
    assert peak > 1000.0 and source in ("measured", "fallback")
