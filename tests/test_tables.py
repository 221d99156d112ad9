"""Host FP64 table builder (librtmc) vs the NumPy/SciPy restatement of
MaterialClass.prepareSigma / prepareSigmaOne, and the solid/air Zoeppritz table."""
import math

import numpy as np
import pytest

from oracle import tables_ref as TR
from radiativetransfermontecarlo_gb300 import MaterialClass, _lib

U = np.random.default_rng(3).random(20000)


def _check(mat, d, ref, n_tab, tol_theta=1e-8):
    MaterialClass.prepareSigma(mat, d)
    for i in range(n_tab):
        c, t = mat.invcdf.knots(i)
        rc, rt = ref["tables"][i]
        assert abs(c.size - rc.size) <= 2, (i, c.size, rc.size)
        assert np.max(np.abs(mat.invcdf.eval(i, U) - TR.invcdf(rc, rt, U))) < tol_theta
    S = np.atleast_1d(mat.Sigma).ravel()
    assert np.allclose(S, np.atleast_1d(ref["Sigma"]).ravel(), rtol=1e-9)


def test_c1_acoustic_exp_matches_numpy_and_recorded_figures():
    geo = {"dimension": 3}
    m = MaterialClass(geo, 10, True, 1, [0.05, 0.05], 0, "exp", 0.1)
    ref = TR.prepare_sigma(3, True, 10, 1.0, [0.05, 0.05], 0.0, "exp", 0.1)
    _check(m, 3, ref, 1)
    assert m.invcdf.info().n_knots[0] == 908390
    assert math.isclose(m.Sigma, 0.4854, rel_tol=1e-3)
    assert math.isclose(m.meanFreeTime, 2.060, rel_tol=1e-3)
    assert math.isclose(m.g, 0.901, rel_tol=1e-3)


def test_c2_elastic_gauss_matches_numpy_and_recorded_figures():
    geo = {"dimension": 3}
    m = MaterialClass(geo, 5, False, [2, 1.155], [0.1, 0.1, 0.1], [0, 0, 0], "gauss", 0.2)
    assert m.SpectralLaw == "gaussian"
    ref = TR.prepare_sigma(3, False, 5, [2, 1.155], [0.1, 0.1, 0.1], [0, 0, 0], "gaussian", 0.2)
    _check(m, 3, ref, 4)
    kn = [m.invcdf.info().n_knots[i] for i in range(4)]
    assert [round(k, -3) for k in kn] == [665000, 553000, 553000, 376000]
    assert np.allclose(m.meanFreeTime, [1.816, 0.876], rtol=2e-3)
    assert math.isclose(m.P2P, 0.687, rel_tol=2e-3) and math.isclose(m.S2S, 0.985, rel_tol=2e-3)
    assert np.allclose(m.P2P, ref["P2P"]) and np.allclose(m.Diffusivity, ref["Diffusivity"])
    assert np.allclose(m.transportMeanFreePath, ref["transportMeanFreePath"])


def test_c3_elastic_2d_exp_matches_numpy():
    geo = {"dimension": 2}
    m = MaterialClass(geo, 8, False, [2, 1.155], [0.2, 0.2, 0.2], [0, 0, 0], "exp", 0.5)
    ref = TR.prepare_sigma(2, False, 8, [2, 1.155], [0.2, 0.2, 0.2], [0, 0, 0], "exp", 0.5)
    _check(m, 2, ref, 4)
    assert np.allclose(m.meanFreeTime, [0.0730, 0.0330], rtol=3e-3)


@pytest.mark.parametrize("acf,d,nu", [("power_law", 3, None), ("VonKarman", 3, 0.3), ("VonKarman", 2, 0.5),
                                      ("triangular", 3, None), ("low_pass", 3, None), ("gaussian", 2, None)])
def test_other_psdf_families(acf, d, nu):
    geo = {"dimension": d}
    m = MaterialClass(geo, 4, True, 1.5, [0.1, 0.05], 0.2, acf, 0.3)
    if nu is not None:
        m.SpectralParam = {"nu": nu}
    ref = TR.prepare_sigma(d, True, 4, 1.5, [0.1, 0.05], 0.2, acf, 0.3, nu=nu)
    _check(m, d, ref, 1, tol_theta=1e-6)


def test_constant_sigma_preset():
    m = MaterialClass.preset(1)  # sigma = 1/(4 pi), v = 2: Sigma = 1 in 3D
    MaterialClass.prepareSigma(m, 3)
    assert math.isclose(m.Sigma, 1.0, rel_tol=1e-12)
    assert math.isclose(m.meanFreeTime, 1.0, rel_tol=1e-12)
    # isotropic: theta = acos(1 - 2u) up to the table's linear interpolation
    th = m.invcdf.eval(0, U)
    assert np.max(np.abs(th - np.arccos(1 - 2 * np.clip(U, 0, 1)))) < 2e-3


def test_validatestring_like_matlab():
    geo = {"dimension": 3}
    for law, want in (("gauss", "gaussian"), ("Exp", "exp"), ("von", "VonKarman"), ("power", "power_law")):
        assert MaterialClass(geo, 1, True, 1, [0.1, 0.1], 0, law, 1).SpectralLaw == want
    with pytest.raises(ValueError):
        MaterialClass(geo, 1, True, 1, [0.1, 0.1], 0, "nonsense", 1)


@pytest.mark.parametrize("vp,vs,rho", [(2.0, 1.155, 1000.0), (2500.0, 2500 / math.sqrt(3), 2000.0), (6.0, 3.4641, 1.0)])
def test_zoeppritz_fluid_matches_numpy_and_conserves_energy(vp, vs, rho):
    ang = np.linspace(0, 90, 181)
    a = _lib.zoeppritz_fluid(ang, vp, vs, rho)
    b = TR.zoeppritz_fluid(ang, vp, vs, rho)
    for k in ("E_Rpp", "E_Rpsv", "E_Tpp", "E_Rsvsv", "E_Rsp", "E_Tsp", "E_Rsh"):
        ok = np.isfinite(b[k])
        assert np.allclose(a[k][ok], b[k][ok], rtol=1e-9, atol=1e-12), k
    tot = a["E_Rpp"] + a["E_Rpsv"] + a["E_Tpp"]
    assert np.allclose(tot[:-1], 1.0, atol=1e-9)  # P incidence energy balance (90 deg excluded)
    assert a["E_Rpsv"][0] == 0.0 and np.all(a["E_Rsh"] == 1.0)


def test_zoeppritz_rejects_solid_lower_medium():
    with pytest.raises(_lib.RtmcError):
        _lib.zoeppritz_fluid([0.0, 10.0], 2.0, 1.0, 1.0, 3.0, 1.0, 1.0)
