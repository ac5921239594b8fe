"""The bench's FP64 closed-form Poisson solve (the reference for the
isolated-solve errors) agrees with the oracle's FP64 solve to rounding, and the
isolated-solve density map has the stated composition."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


@pytest.mark.parametrize("m,n,bw,bh", [(32, 64, 1.0, 1.0), (64, 32, 0.9, 1.7), (128, 128, 1.3, 1.1)])
def test_fp64_closed_form_matches_oracle(built, m, n, bw, bh):
    pytest.importorskip("scipy")
    import bench
    from oracle import erp_oracle as O
    rng = np.random.default_rng(m + 3 * n)
    rho = (0.5 + rng.random((m, n))).astype(np.float32)
    got = bench.poisson_fp64(rho, bw, bh)
    want = O.poisson(rho, bw, bh, dtype=np.float64)
    for g, w in zip(got, want):
        assert np.linalg.norm(g - w) / np.linalg.norm(w) < 1e-12


def test_spectral_workload_map(built):
    import reda_erplacer_gb300 as R
    a = R.workload_spectral(512, seed=5)
    b = R.workload_spectral(512, seed=5)
    assert a.dtype == np.float32 and a.shape == (512, 512)
    assert np.array_equal(a, b)                      # seeded
    assert a.min() >= 0.7 - 1e-6                     # background + non-negative blobs
    assert np.count_nonzero(a == 1.0) > 10 * 16 * 16  # ten macro blocks of >= side/32 squared


def test_bench_workloads_are_the_package_workloads(built):
    """bench.py keeps its own copy of the workload definitions (the reference
    arm must not import the package); it equals the package's."""
    import bench
    import reda_erplacer_gb300 as R
    assert bench.WORKLOADS == R.design.WORKLOADS


def test_reference_arm_generator_builds_the_same_design(built):
    """The generator compiled on its own (oracle/_build/liberp_synth.so, which
    the reference arm uses) gives the product generator's design bit for bit."""
    import reda_erplacer_gb300 as R
    from oracle import erp_oracle as O
    args, _ = R.design.WORKLOADS["small"]
    a, b = O.synth(**args), R.synth(**args)
    for k, va in vars(a).items():
        vb = getattr(b, k)
        assert (np.array_equal(va, vb) if isinstance(va, np.ndarray) else va == vb), k


def test_parity_summary_fields():
    import bench
    gpu = [(100.0, 0.9), (110.0, 0.5), (120.0, 0.09), (125.0, 0.05), (130.0, 0.2)]
    ref = [(100.0, 0.9), (111.0, 0.5), (119.0, 0.1), (126.0, 0.06), (128.0, 0.3)]
    p = bench.parity_summary(gpu, ref, 3)
    assert p["iterations"] == 5
    assert p["at_overflow_0.10"]["iteration"] == 3
    assert abs(p["at_overflow_0.10"]["hpwl_rel"] - (120.0 - 119.0) / 119.0) < 1e-12
    assert p["overflow_min"]["iteration_gpu"] == 4 and p["overflow_min"]["iteration_ref"] == 4
    assert abs(p["last"]["overflow_abs"] - (0.2 - 0.3)) < 1e-12
