"""The bench line's roofline objects on CPU: DRAM traffic comes from the committed
ncu summaries under profiles/ (a machine-readable `dram_bytes_per_launch_scaled:`
line each), and the fractions the line reports as `frac` are DRAM-side, so they
stay below the measured copy bandwidth for the step times the summaries record.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

PEAK = 6690.8  # GB/s, the measured copy bandwidth of the GB300s


@pytest.mark.parametrize("name", ["plain_batch_kernel_rmat20.txt", "staged_kernel_batched512.txt",
                                  "spmm_kernel_rmat20.txt", "sparse_embedding_rmat20.txt"])
def test_profiles_carry_dram_traffic(name):
    t = bench.profile_traffic(name)
    assert t is not None and t > 0


def test_missing_profile_gives_none():
    assert bench.profile_traffic("no_such_profile.txt") is None


def test_spmm_roofline_is_dram_side():
    # the SpMM step at R-MAT s20, D=128: 1.65 ms, 17.8 GB of gathered rows
    r = bench.spmm_roofline(17824664528, 2281497552, 1.65e-3, PEAK, "measured")
    assert r["traffic"] == bench.profile_traffic("spmm_kernel_rmat20.txt")
    assert 0.2 < r["frac"] < 1.0
    assert r["frac_gathered"] > 1.0  # hub rows come from L2: the gathered figure passes the peak
    assert r["achieved"] == pytest.approx(r["traffic"] / 1.65e-3 / 1e9)


def test_sparse_roofline_is_dram_side():
    # the sparse-embedding step: 13.09 ms, 97.6 GB of gathered rows
    r = bench.sparse_roofline(97.6e9, 13.09e-3, PEAK, "measured")
    assert 0.2 < r["frac"] < 1.0
    assert r["frac_gathered"] > 1.0
