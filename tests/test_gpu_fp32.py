"""The FP32 update mode (fim_opts.fp32_update): triangle, tet and edge
candidates take their FP32 value wherever the running-error screen is
conclusive, FP64 only where it is not.  Measured on the GB300 against the
FP64 oracle: within 1e-4 max(t) on the isotropic unit cube, but not on the
anisotropic slab, where the reference's freeze rule turns float rounding
into errors of a few 1e-2 of max(t) (0.5 on the 1M-vertex slab) -- which
is why the default solve stays bit-exact FP64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F(built_library):
    import fim_api
    return fim_api


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def _oracle(O, c):
    nV = c["xyz"].shape[0]
    slots, _, _, _ = O.reference_slots(nV, c["tets"], None)
    geo = O.metric_geo(slots, c["xyz"], c["fib"], c["cf"], c["ct"])
    phi, st, it, _ = O.solve_pure(nV, slots, geo, c["seed_v"], c["seed_t"])
    return phi, st, it


def _err(phi, phi_o):
    r = phi_o < 1e300
    return np.abs(phi - phi_o)[r] / phi_o[r].max()


def test_fp32_cube_within_tolerance(F, O):
    import fim_mesh
    c = fim_mesh.cube_case(20)
    phi_o, _, _ = _oracle(O, c)
    phi, _, st = F.solve_case(c, fp32_update=1)
    _, _, st64 = F.solve_case(c)
    assert np.array_equal(phi < F.INF, phi_o < 1e300)
    assert _err(phi, phi_o).max() <= 1e-4
    assert st["exact_evals"] < st64["exact_evals"] / 4  # most solves stay in FP32


def test_fp32_slab_error_reported(F, O):
    """The anisotropic slab runs and converges in FP32 mode, with an error
    above the FP64 path's zero but bounded (a few 1e-2 of max(t) here)."""
    import fim_mesh
    c = fim_mesh.slab_case(cells=(66, 23, 10))
    phi_o, _, _ = _oracle(O, c)
    phi, _, st = F.solve_case(c, fp32_update=1)
    e = _err(phi, phi_o)
    assert np.array_equal(phi < F.INF, phi_o < 1e300)
    assert 0.0 < e.max() < 0.1 and np.sqrt(np.mean(e ** 2)) < 1e-3
