"""Host-side pieces of bench.py that need no GPU: the batched workload's CPU
baseline (oracle port in a spawn process pool, sample scaled to the whole
batch)."""
import os
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpu_baseline_batch_small_sample():
    sys.path.insert(0, REPO)
    import bench
    cb = bench.cpu_baseline_batch([1000, 1001], 1e-8, 256, workers=2)
    assert cb["kind"] == "port" and cb["unit"] == "s" and cb["cores"] == 2
    assert cb["all_converged"] and cb["iterations_max"] > 0
    # the sample's wall time scaled by 256 / 2
    assert cb["value"] > 0 and "2 of 256 instances" in cb["sample"]
