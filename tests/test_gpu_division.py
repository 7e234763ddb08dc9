"""The kernels divide by |n| and by 3 with a correctly rounded reciprocal and
one FMA correction (Markstein's theorem) instead of IEEE division; the face
terms are only bit-identical to the reference arithmetic if that gives the
IEEE result.  x/3 is checked for every float, x/b on random pairs."""
import pytest

pytestmark = pytest.mark.gpu


def test_fma_corrected_division_matches_ieee(hctx):
    bad = hctx.division_check(n_pairs=1 << 28, seed=12345)
    assert bad == [0, 0, 0], bad
