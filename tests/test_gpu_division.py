"""Arithmetic that the kernels use in place of plain IEEE FP32 operations:

* x/|n| and x/3 by a correctly rounded reciprocal plus one FMA correction
  (Markstein's theorem) -- x/3 checked for every float, x/b on random pairs;
* Blackwell's packed add/sub/mul/fma.rn.f32x2 for two faces at a time --
  each half checked against the scalar IEEE op on random operands.

The face terms are only bit-identical to the reference arithmetic if both
give the IEEE result."""
import pytest

pytestmark = pytest.mark.gpu


def test_fma_corrected_division_matches_ieee(hctx):
    bad = hctx.division_check(n_pairs=1 << 28, seed=12345)
    assert bad == [0, 0, 0], bad


def test_packed_fp32_ops_match_scalar_ieee(hctx):
    div, packed, ex = hctx.arith_check(n_pairs=1 << 26, seed=777)
    assert div == [0, 0, 0], div
    assert packed == [0, 0, 0, 0], (packed, ex)
