"""The FP64 issue structure of the GPU the solver kernels are designed around
(measured by the probe library): every SM sub-partition retires one FP64
warp instruction at a time at a fixed rate, masked-off lanes cost as much as
active ones, and one warp with a single dependency chain per sub-partition
already reaches the SM's FP64 peak.  These facts are why divergence and tails
cost in proportion, why trajectories-per-thread and extra warps add nothing
for the FP64 pipe, and why a small ensemble (fewer warps than sub-partitions)
cannot reach the peak."""
import pytest

pytestmark = pytest.mark.gpu


def test_fp64_issue_structure(pkg):
    r = pkg._lib.probe_fp64_issue(0)
    full = r["full_32_lanes"]
    # masked lanes: the same warp-instruction rate with 8 of 32 lanes active
    assert abs(r["full_8_lanes"] / full - 1) < 0.05
    # one warp per sub-partition with one chain reaches the full-occupancy rate
    assert r["one_warp_per_smsp"] / full > 0.9
    # a lone warp gets a quarter of the SM (one sub-partition), with or without instruction-level parallelism
    assert 0.2 < r["one_warp_1_chain"] / full < 0.3
    assert abs(r["one_warp_8_chains"] / r["one_warp_1_chain"] - 1) < 0.1
