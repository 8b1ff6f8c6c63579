"""Host logic of bench.py (CPU only): the radices the kernels run, the FP64 operation model behind the
roofline's `fp64` figures, the grid-point count of the metric with and without bands, and the whole-job value."""
import pytest

import bench


def test_stage_radices_follow_the_plan_builder():
    # 4s first (the first stage needs no twiddles), then 2s, then 3s (the z-forward prunes the last one)
    assert bench._stages(576) == [4, 4, 4, 3, 3]
    assert bench._stages(432) == [4, 4, 3, 3, 3]
    assert bench._stages(384) == [4, 4, 4, 2, 3]
    assert bench._stages(144) == [4, 4, 3, 3]
    assert bench._stages(6) == [2, 3]


def test_fft_operation_model():
    # one radix-4 butterfly without twiddles: 16 real additions
    assert bench.fft_flops(4) == 16.0
    # length 12 = radix 4 (3 butterflies, no twiddles) then radix 3 (4 butterflies with twiddles, 32 each)
    assert bench.fft_flops(12) == 3 * 16 + 4 * 32
    # a pruned last radix-3 stage skips the middle output: 28 instead of 32 per butterfly
    assert bench.fft_flops(12, prune_last=True) == 3 * 16 + 4 * 28


def test_product_pass_model_at_configuration_2():
    # the model figure the bench line reports per product-pass launch at configuration 2 (448 interior levels,
    # 576 z rows, 193 kept kx modes)
    assert bench.xprod_flops(576, 576, 193, 448) == pytest.approx(35.303e9, rel=1e-4)


def test_grid_points_with_and_without_bands():
    cfg = dict(ngalx=576, ngalz=576)
    assert bench.grid_points(cfg, 452, None) == 576 * 576 * 452
    # bands: the middle band's levels N(4,1)+1 .. N(4,2) count the middle band's own points
    N = [0] * 20
    N[1 * 4 + 3], N[2 * 4 + 3] = 100, 350  # N(4,1), N(4,2)
    banded = dict(cfg, ngalx2=384, ngalz2=384)
    assert bench.grid_points(banded, 452, N) == 576 * 576 * (452 - 250) + 384 * 384 * 250


def test_whole_job_value_sums_the_replicas():
    # points x steps / seconds, times the number of replicas
    assert bench.whole_job_value(1, 1000, 4, 2.0) == pytest.approx(1000 * 4 / 2e-3)
    assert bench.whole_job_value(8, 1000, 4, 2.0) == pytest.approx(8 * 1000 * 4 / 2e-3)
