"""The byte model behind bench.py's roofline (CPU): per-launch algorithmic bytes of each pass
from the compact layout (kept modes only), the 6.08 GB step total at 256^3 quoted beside the
measured step rate, and the MHD variant."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_hydro_256_pass_bytes():
    import bench
    n, K, c = 256, 85, 8
    M, Hk = 2 * K + 1, K + 1
    X, Y, S = n * M * Hk * c, n * n * Hk * c, M * M * Hk * c
    b = bench.algorithmic_bytes(n)
    assert b["ky_inverse"] == 6 * (X + Y) == 451_239_936
    assert b["ky_forward"] == 3 * (X + Y) == 225_619_968
    assert b["kz_product_hd"] == 9 * Y == 405_798_912
    # x stage, mean over the four RK4 stages: W, S (and acc from stage 2) in, acc (S at stage 4)
    # and the six inverse-x fields out
    assert b["kx_stage_hd"] == pytest.approx(9 * X + 8.25 * S) == 437_032_908
    step = 4 * sum(b.values())
    assert step == pytest.approx(6.0788e9, rel=1e-4)


def test_mhd_pass_bytes_scale_with_the_field_counts():
    import bench
    h, m = bench.algorithmic_bytes(128), bench.algorithmic_bytes(128, F=6)
    assert m["ky_inverse"] == 2 * h["ky_inverse"]
    assert m["ky_forward"] == 2 * h["ky_forward"]
    assert m["kz_product_mhd"] == 2 * h["kz_product_hd"]
    assert m["kx_stage_mhd"] == pytest.approx(2 * h["kx_stage_hd"])


def test_reduced_cutoff_moves_fewer_bytes():
    import bench
    full, cut = bench.algorithmic_bytes(64), bench.algorithmic_bytes(64, K=10)
    assert all(cut[k] < full[k] for k in full)
