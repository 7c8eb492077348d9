"""GroupwiseRegistration oracle: the reference's own kernels run on the host
(oracle/refkernels/registration_host.hpp) against the committed fixtures, and
the geometry the registration derives from its parameters."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402
from oracle import refkernels as K  # noqa: E402

CASES = [c[0] for c in make_golden.REG_CASES]


def _load(name):
    return dict(np.load(os.path.join(HERE, "golden", name)))


def _prm(d):
    return {k[4:]: (tuple(d[k]) if d[k].ndim else d[k].item()) for k in d if k.startswith("prm_")}


@pytest.mark.parametrize("name", CASES)
def test_fixture_inputs_regenerate(name):
    d = _load(name)
    img = make_golden.registration_inputs(int(d["N"]), int(d["F"]), int(d["seed"]))
    np.testing.assert_array_equal(img, d["images"])


@pytest.mark.parametrize("name", CASES)
def test_reference_kernels_reproduce_fixture(name):
    if K.build() is None or not K.available():
        pytest.skip("reference kernel sources unavailable")
    d = _load(name)
    r = K.registration(d["images"], **_prm(d))
    assert r["iterations"] == int(d["iterations"])
    for k in ("T", "xn", "H", "bb"):
        np.testing.assert_array_equal(r[k], d[k], err_msg=k)
    assert r["Wn"] == float(d["Wn"])


def _circle_geometry(N, radius):
    # setMask (GroupwiseRegistration.cpp:486-531): pixels within the radius of
    # the centre ((N+1)/2, 1-based), their count and 1-based bounding box
    j = np.arange(N)
    Cv = (1 - (N + 1) / 2 + j) ** 2
    inside = (Cv[None, :] + Cv[:, None]) <= radius ** 2
    rows, cols = np.nonzero(inside)
    return int(inside.sum()), [cols.min() + 1, rows.min() + 1, cols.max() + 1, rows.max() + 1]


@pytest.mark.parametrize("name", CASES)
def test_geometry_and_descent(name):
    d = _load(name)
    prm = _prm(d)
    N, F = int(d["N"]), int(d["F"])
    area, bb = _circle_geometry(N, prm["radius"])
    assert int(d["areaX"]) == area
    assert list(d["bb"]) == bb
    # control grid: C = floor((|c - bb| + rp) / Dp) on each side, rp = (E+1) Dp / 2
    c = (bb[0] + bb[2]) / 2
    rp = (prm["E"] + 1) * prm["Dp"][0] // 2
    C = int(np.floor((abs(c - bb[0]) + rp) / prm["Dp"][0]))
    assert int(d["C0"]) == int(d["C1"]) == 2 * C + 1
    assert d["T"].shape == (2, F, 2 * C + 1, 2 * C + 1)
    # outside the bounding box the mesh is the identity
    xn = d["xn"]
    rr, cc = np.meshgrid(np.arange(N), np.arange(N), indexing="ij")
    out = (rr < bb[1] - 1) | (rr > bb[3] - 1) | (cc < bb[0] - 1) | (cc > bb[2] - 1)
    for f in range(F):
        np.testing.assert_array_equal(xn[0, f][out], (cc + 1)[out])
        np.testing.assert_array_equal(xn[1, f][out], (rr + 1)[out])
    # the step sizes of the fixtures make the metric fall overall
    H = d["H"]
    assert H[-1] < H[0]
    assert len(H) == int(d["iterations"]) + 1


@pytest.mark.parametrize("name", CASES)
def test_restatement_matches_reference_kernels(name):
    """oracle/registration.py (the algorithm per quantity, the reference's
    regularisation gradient included) against the fixtures of the reference's
    own kernels: same iterations and weight, T and xn to a few float ulps."""
    from oracle import registration as RG
    d = _load(name)
    prm = _prm(d)
    r = RG.Registration(int(d["N"]), int(d["F"]), **prm).run(d["images"])
    assert r["iterations"] == int(d["iterations"])
    assert r["Wn"] == pytest.approx(float(d["Wn"]), rel=1e-6)
    scale = np.abs(d["T"]).max()
    # a few float roundings that the projection (dH - mean) amplifies over the iterations
    assert np.abs(r["T"] - d["T"]).max() <= make_golden.REG_T_TOL.get(name, 5e-6) * scale + 1e-6
    assert np.abs(r["xn"] - d["xn"]).max() <= make_golden.REG_XN_TOL.get(name, 2e-5)
    np.testing.assert_allclose(r["H"], d["H"], rtol=make_golden.REG_H_TOL.get(name, 2e-6))


def test_restatement_starting_displacements():
    """A later motion iteration starts from the previous T (optimizer.cpp:
    TData given): the restatement against the reference kernels, both
    continuing from the T of a first run."""
    if K.build() is None or not K.available():
        pytest.skip("reference kernel sources unavailable")
    from oracle import registration as RG
    d = _load(CASES[0])
    prm = dict(_prm(d), nmax=3)
    T0 = d["T"]
    ref = K.registration(d["images"], T_init=T0, **prm)
    r = RG.Registration(int(d["N"]), int(d["F"]), **prm).run(d["images"], T_init=T0)
    assert r["iterations"] == ref["iterations"]
    assert np.abs(r["T"] - ref["T"]).max() <= 2e-6 * np.abs(ref["T"]).max() + 1e-6
    np.testing.assert_allclose(r["H"], ref["H"], rtol=2e-6)
    assert r["H"][0] == ref["H"][0] == d["H"][0]  # the metric restarts from the unregistered frames


@pytest.mark.parametrize("N,F,radius,E", [(64, 4, 12, 3), (64, 5, 14, 3), (96, 6, 20, 3), (256, 20, 40, 3),
                                          (128, 3, 30, 3), (64, 4, 12, 1), (64, 4, 12, 2), (256, 20, 40, 2)])
def test_library_geometry_matches_restatement(built_lib, N, F, radius, E):
    """gbn_registration_info_get (host code of the library, no GPU needed):
    control grid, bounding box and region-of-interest area as the restatement
    derives them from init() and creabspline()."""
    from opencliper_gb300 import api
    from oracle import registration as RG
    info = api.registration_info(N, F, api.registration_params(radius=radius, E=E))
    g = RG.Geometry(N, F, radius, E)
    assert info["cp"] == g.Cp
    assert info["bound_box"] == g.bb
    assert info["area"] == g.areaX


@pytest.mark.parametrize("over,code", [(dict(radius=0), -2), (dict(E=4), -2), (dict(Dp=(4, 3)), -2),
                                       (dict(nmax=0), -1), (dict(radius=31), -2)])
def test_library_refuses_geometry(built_lib, over, code):
    """Refusals, without a GPU: the whole-box region (degenerate in the
    reference), other spline orders, unequal spacing, nmax 0, and a grid whose
    supports leave a 64 x 64 image."""
    from opencliper_gb300 import api
    from opencliper_gb300._abi import GbnError
    with pytest.raises(GbnError) as e:
        api.registration_info(64, 4, api.registration_params(**over))
    assert e.value.code == code
