"""Headless point rendering in place of the reference's OpenGL viewer
(StellarSolverVisualizer.cpp:4-20, 208-253): the oracle's restatement on known
points, and the engine's bh_render byte for byte against it."""
import numpy as np
import pytest


def test_oracle_render_known_points(oracle):
    # 10 x 10 pixels over [0, 10]^2: pixel (col, row-from-bottom) = floor(x), floor(y)
    x = np.array([0.5, 0.5, 0.5, 9.99, 10.0, -0.01, 3.2] + [7.5] * 60, np.float32)
    y = np.array([0.5, 0.5, 0.5, 9.99, 5.0, 5.0, 8.7] + [2.5] * 60, np.float32)
    img = oracle.render(x, y, 10, 10, (0.0, 10.0, 0.0, 10.0))
    assert img.shape == (10, 10, 4)
    def px(col, row_from_bottom):
        return tuple(int(v) for v in img[9 - row_from_bottom, col])
    assert px(0, 0) == (77, 77, 77, 135)    # 3 points: 0.3 -> 76.5 -> 77; alpha 0.53 -> 135.15
    assert px(9, 9) == (26, 26, 26, 130)    # 1 point: 25.5 -> 26 (half up); alpha 0.51 -> 130.05
    assert px(3, 8) == (26, 26, 26, 130)
    assert px(7, 2) == (255, 255, 255, 255)  # 60 points saturate colour and alpha
    assert px(5, 5) == (0, 0, 0, 128)        # background: (0, 0, 0, 0.5)
    hit = (img[..., 0] > 0).sum()
    assert hit == 4                          # (10, 5) and (-0.01, 5) fall outside


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["plain", "mixed"])
def test_engine_render_matches_oracle(oracle, mode):
    from stellarsolver_gb300 import bh, models

    x, y, vx, vy, m = models.disk(1 << 16, 0x5EED6000)
    with bh.BarnesHutSystem(len(x), mode=mode, eps2=0.01, timestep=1e-3) as s:
        s.set_state(x, y, vx, vy, m)
        s.step(3)
        img = s.render()
        small = s.render(320, 200, (-60.0, 60.0, -40.0, 40.0))
        xh, _, yh, _ = s.get_positions_hilo()
    assert np.array_equal(img, oracle.render(xh, yh))
    assert np.array_equal(small, oracle.render(xh, yh, 320, 200, (-60.0, 60.0, -40.0, 40.0)))
    assert (img[..., 0] > 0).sum() > 1000
