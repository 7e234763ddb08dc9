"""The CPU restatement of the surrogate network checks itself: analytic
gradients against central differences (FP64), and the bfloat16 rounding
helper against the definition of round-to-nearest-even."""
import numpy as np

from oracle import mlp


def _net(rng, dims):
    Ws = [rng.normal(0, 1.0 / np.sqrt(k), (k, n)) for k, n in dims]
    bs = [rng.normal(0, 0.1, n) for _, n in dims]
    return Ws, bs


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    dims = [(8, 16), (16, 16), (16, 16), (16, 8)]
    Ws, bs = _net(rng, dims)
    x = rng.normal(size=(32, 8))
    t = rng.normal(size=(32, 6))
    for layer, a, n in mlp.finite_difference(x, Ws, bs, t, 6, n_probe=12):
        assert abs(a - n) <= 1e-7 + 1e-5 * abs(n), (layer, a, n)


def test_bias_gradient_is_column_sum_of_output_gradient():
    rng = np.random.default_rng(1)
    dims = [(4, 8), (8, 8), (8, 8), (8, 4)]
    Ws, bs = _net(rng, dims)
    x = rng.normal(size=(16, 4))
    t = rng.normal(size=(16, 3))
    eps = 1e-6
    _, dbs = mlp.backward(x, Ws, bs, t, 3)
    for l in range(4):
        for j in range(dims[l][1]):
            bp = [b.copy() for b in bs]
            bm = [b.copy() for b in bs]
            bp[l][j] += eps
            bm[l][j] -= eps
            num = (mlp.loss(mlp.forward(x, Ws, bp)[0][-1], t, 3) - mlp.loss(mlp.forward(x, Ws, bm)[0][-1], t, 3)) / (2 * eps)
            assert abs(dbs[l][j] - num) <= 1e-7 + 1e-5 * abs(num)


def test_bf16_round_to_nearest_even():
    vals = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -9, 1.0 + 2.0 ** -9, -2.5, 3.0e-39, 65504.0],
                    dtype=np.float32)
    r = mlp.bf16_round(vals)
    # 1 + 2^-9 is a tie between 1 and 1 + 2^-7 -> even (1); 1 + 3*2^-9 rounds up
    assert r[0] == 1.0 and r[3] == 1.0
    assert r[2] == np.float32(1.0 + 2.0 ** -7)
    assert r[4] == -2.5
    bits = r.view(np.uint32)
    assert np.all(bits & 0xFFFF == 0)
    back = mlp.bf16_bits_to_f32((bits >> 16).astype(np.uint16))
    assert np.array_equal(back, r)
