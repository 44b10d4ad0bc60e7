"""The CPU conv oracle is self-consistent (adjoint identities), CPU only."""
import numpy as np

from oracle import conv_ref


def test_dgrad_and_wgrad_are_adjoints_of_conv():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((4, 5, 6, 3))
    w = rng.standard_normal((27, 2, 3))
    dy = rng.standard_normal((4, 5, 6, 2))
    y = conv_ref.conv3d(x, w)
    # <conv(x, w), dy> == <x, dgrad(dy, w)> == <w, wgrad(x, dy)>
    lhs = np.sum(y * dy)
    assert abs(lhs - np.sum(x * conv_ref.conv3d_dgrad(dy, w))) < 1e-9 * abs(lhs)
    assert abs(lhs - np.sum(w * conv_ref.conv3d_wgrad(x, dy))) < 1e-9 * abs(lhs)


def test_center_tap_is_pointwise_matmul():
    rng = np.random.default_rng(1)
    x = rng.standard_normal((3, 3, 3, 4))
    w = np.zeros((27, 5, 4))
    w[13] = rng.standard_normal((5, 4))
    assert np.allclose(conv_ref.conv3d(x, w), x @ w[13].T)


def test_bf16_round_is_exactly_representable():
    a = np.array([1.0, 1.00390625, 3.14159, -2.5e-3], np.float32)
    r = conv_ref.bf16_round(a)
    assert np.all((r.view(np.uint32) & 0xFFFF) == 0)
    assert r[0] == 1.0 and r[1] == 1.0  # ties to even
