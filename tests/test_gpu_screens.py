"""The FP32 screens against the FP64 local solves they bound, on random
corners (fim_selftest_screens): every bound must hold, or the solve would
not be bit-exact.  The random corners reach both the value paths and the
early exits of the screens."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F(built_library):
    import fim_api
    return fim_api


@pytest.mark.parametrize("seed", [1, 2])
def test_screens_bound_the_fp64_solves(F, seed):
    r = F.selftest_screens(1 << 24, seed=seed)
    assert r["tets"] == 1 << 24 and r["tris"] == 3 << 24
    assert r["tet_violations"] == 0, r
    assert r["tri_violations"] == 0, r
    # both paths are exercised: solves with a value and without
    assert 0.01 * r["tets"] < r["tets_with_value"] < 0.99 * r["tets"], r
    assert 0.01 * r["tris"] < r["tris_with_value"] < 0.99 * r["tris"], r
