"""NumPy/SciPy restatement of the reference's FP64 table builders.

TEST INFRASTRUCTURE ONLY: used by tests/ to check the product library's C++ table
builder, never by the product path.

Restates, from cottereau/RadiativeTransferMonteCarlo:
  * the normalised power spectral densities Phi(z) of @MaterialClass/MaterialClass.m
    (Exponential :479-517, PowerLaw :519-558, Gaussian :560-599, Triangular :601-630,
    LowPass :632-662, VonKarman :664-710);
  * the isotropic differential cross-sections sigma(theta) of calcSigmaIsotropic
    (MaterialClass.m:172-359): acoustic 2D/3D (:200-236), elastic 2D P-SV (:258-310)
    and elastic 3D (:311-356);
  * prepareSigmaOne (MaterialClass.m:2443-2463): Sigma and Sigma' by adaptive
    quadrature (MATLAB `integral`; here scipy.integrate.quad), the 1e6-point pdf, the
    cumsum cdf scaled by pi/Nth, the diff(cdf) > 1e-8 knot filter and the linear
    griddedInterpolant with linear extrapolation;
  * prepareSigma (MaterialClass.m:2379-2442): mean free times, P2P, S2S, transport
    mean free paths and diffusivity;
  * ZoeppritzFluid (@MaterialClass/ZoeppritzFluid.m:1-244) for the solid/air table of
    MaterialClass.Zoeppritz (MaterialClass.m:1786-1885), with complex arithmetic where
    asin of an argument above 1 turns the angles complex.
"""
from __future__ import annotations

import math

import numpy as np
from scipy import integrate, special

PSDF_NAMES = ("exp", "gaussian", "power_law", "triangular", "low_pass", "VonKarman")


def _heaviside(h):
    h = np.asarray(h, dtype=float)
    return np.where(h > 0, 1.0, np.where(h == 0, 0.5, 0.0))


def psdf(name: str, d: int, nu: float | None = None):
    """Return Phi(z) for PSDF family `name` in dimension d (MaterialClass.m:479-710)."""
    if name == "exp":
        if d == 2:
            a = math.sqrt(2.0)
            return lambda z: 1.0 / (4 * np.pi * (1 + (z / a) ** 2) ** 1.5)
        a = 6.0 ** (1.0 / 3.0)
        return lambda z: 1.0 / (6 * np.pi ** 2 * (1 + (z / a) ** 2) ** 2)
    if name == "gaussian":
        if d == 2:
            return lambda z: 1.0 / (4 * np.pi) * np.exp(-z ** 2 / 4)
        a = (3 * math.sqrt(math.pi) / 4) ** (2.0 / 3.0)
        return lambda z: 1.0 / (6 * np.pi ** 2) * np.exp(-z ** 2 / (4 * a))
    if name == "power_law":
        if d == 2:
            return lambda z: z * special.k1(z) / (4 * np.pi)
        a = (3 * math.pi / 4) ** (1.0 / 3.0)
        return lambda z: 1.0 / (6 * np.pi ** 2) * np.exp(-z / a)
    if name == "triangular":
        assert d == 3
        return lambda z: (3 / 8 / np.pi ** 4) * (1 - z / 2 / np.pi) * _heaviside(2 * np.pi - z)
    if name == "low_pass":
        assert d == 3
        a = 3 * math.pi / 2
        return lambda z: (2 / 9 / np.pi ** 4) * _heaviside(a - z)
    if name == "VonKarman":
        assert nu is not None
        if d == 2:
            a = 2 * math.sqrt(nu)
            return lambda z: 1 / (4 * np.pi) / (1 + (z / a) ** 2) ** (nu + 1)
        a = (6 * math.sqrt(math.pi) * math.gamma(nu + 1.5) / math.gamma(nu)) ** (1.0 / 3.0)
        return lambda z: 1 / (6 * np.pi ** 2) / (1 + (z / a) ** 2) ** (nu + 1.5)
    raise ValueError(name)


def sigma_functions(d, acoustics, freq, v, cv, corr, acf, lc, nu=None):
    """Differential cross-sections (MaterialClass.m:172-359); returns [s] or [[s11,s12],[s21,s22]]."""
    Phi = psdf(acf, d, nu)
    omega = 2 * np.pi * freq
    if acoustics:
        zeta = omega / v * lc
        dkk, drr = cv[0], cv[1]
        rkr = corr if np.isscalar(corr) else corr[0]
        p = zeta ** 2 if d == 2 else zeta ** 3

        def s(th):
            c = np.cos(th)
            return (np.pi / 2) * omega * p * (c ** 2 * drr ** 2 + 2 * c * rkr * dkk * drr + dkk ** 2) \
                * Phi(zeta * np.sqrt(2 * (1 - c)))
        return [s]
    vp, vs = v
    K = vp / vs
    zP = omega / vp * lc
    zS = K * zP
    dll, dmm, drr = cv
    rlm, rlr, rmr = corr
    if d == 2:
        def sPP(th):
            c = np.cos(th)
            return (np.pi / 2) * omega * zP ** 2 * (
                (1 - 2 / K ** 2) ** 2 * dll ** 2 + 4 * (1 / K ** 2 - 2 / K ** 4) * rlm * dll * dmm * c ** 2
                + (4 / K ** 4) * dmm ** 2 * c ** 4 + drr ** 2 * c ** 2
                - 2 * (1 - 2 / K ** 2) * rlr * dll * drr * c - (4 / K ** 2) * rmr * dmm * drr * c ** 3) \
                * Phi(zP * np.sqrt(2 * (1 - c)))

        def sPS(th):
            c = np.cos(th)
            return (np.pi / 2) * omega * zP ** 2 * (K ** 2 * drr ** 2 + 4 * dmm ** 2 * c ** 2
                                                  - 4 * K * rmr * dmm * drr * c) * (1 - c ** 2) \
                * Phi(zP * np.sqrt(1 + K ** 2 - 2 * K * c))

        def sSP(th):
            c = np.cos(th)
            return (np.pi / 2) * omega * zP ** 2 * (drr ** 2 + (4 / K ** 2) * dmm ** 2 * c ** 2
                                                  - (4 / K) * rmr * dmm * drr * c) * (1 - c ** 2) \
                * Phi(zS * np.sqrt(1 + 1 / K ** 2 - 2 * c / K))

        def sSS(th):
            c = np.cos(th)
            G = 2 * c ** 2 - 1
            return (np.pi / 2) * omega * zS ** 2 * (drr ** 2 * c ** 2 + dmm ** 2 * G ** 2
                                                  - 2 * rmr * dmm * drr * c * G) \
                * Phi(zS * np.sqrt(2 * (1 - c)))
        return [[sPP, sPS], [sSP, sSS]]

    def sPP(th):
        c = np.cos(th)
        return (np.pi / 2) * omega * zP ** 3 * (
            (1 - 2 / K ** 2) ** 2 * dll ** 2 + 4 * (1 / K ** 2 - 2 / K ** 4) * rlm * dll * dmm * c ** 2
            + (4 / K ** 4) * dmm ** 2 * c ** 4 + drr ** 2 * c ** 2
            - 2 * (1 - 2 / K ** 2) * rlr * dll * drr * c - (4 / K ** 2) * rmr * dmm * drr * c ** 3) \
            * Phi(zP * np.sqrt(2 * (1 - c)))

    def sPS(th):
        c = np.cos(th)
        return (np.pi / 2) * K * omega * zP ** 3 * (K ** 2 * drr ** 2 + 4 * dmm ** 2 * c ** 2
                                                  - 4 * K * rmr * dmm * drr * c) * (1 - c ** 2) \
            * Phi(zP * np.sqrt(1 + K ** 2 - 2 * K * c))

    def sSP(th):
        c = np.cos(th)
        return (np.pi / 4 / K ** 3) * omega * zS ** 3 * (drr ** 2 + (4 / K ** 2) * dmm ** 2 * c ** 2
                                                       - (4 / K) * rmr * dmm * drr * c) * (1 - c ** 2) \
            * Phi(zS * np.sqrt(1 + 1 / K ** 2 - 2 / K * c))

    def sSS(th):
        c = np.cos(th)
        ph = Phi(zS * np.sqrt(2 * (1 - c)))
        return (np.pi / 4) * omega * zS ** 3 * (drr ** 2 * (1 + c ** 2) + dmm ** 2 * (4 * c ** 4 - 3 * c ** 2 + 1)
                                               - rmr * dmm * drr * 4 * c ** 3) * ph
    return [[sPP, sPS], [sSP, sSS]]


def prepare_sigma_one(sigma, d, nth=1_000_000, epsrel=1e-12, epsabs=1e-14):
    """prepareSigmaOne (MaterialClass.m:2443-2463) -> (Sigma, Sigma', cdf_knots, theta_knots)."""
    xth = np.linspace(0.0, np.pi, nth)
    f = lambda t: float(sigma(np.float64(t)))
    if d == 2:
        S = 2 * integrate.quad(f, 0, np.pi, epsabs=epsabs, epsrel=epsrel, limit=500)[0]
        Sp = 2 * integrate.quad(lambda t: f(t) * math.cos(t), 0, np.pi, epsabs=epsabs, epsrel=epsrel, limit=500)[0]
        pdf = (2 / S) * sigma(xth)
    else:
        S = 2 * np.pi * integrate.quad(lambda t: f(t) * math.sin(t), 0, np.pi, epsabs=epsabs, epsrel=epsrel,
                                       limit=500)[0]
        Sp = 2 * np.pi * integrate.quad(lambda t: f(t) * math.sin(t) * math.cos(t), 0, np.pi, epsabs=epsabs,
                                        epsrel=epsrel, limit=500)[0]
        pdf = (2 * np.pi / S) * np.sin(xth) * sigma(xth)
    pdf = np.broadcast_to(pdf, xth.shape)
    cdf = np.cumsum(np.nan_to_num(pdf, nan=0.0)) * (np.pi / nth)
    ind = np.nonzero(np.diff(cdf) > 1e-8)[0]
    ind = np.unique(np.concatenate([ind, ind + 1]))
    c, t = cdf[ind], xth[ind]
    keep = np.concatenate([[True], np.diff(c) > 0])  # griddedInterpolant needs strictly increasing knots
    return S, Sp, c[keep], t[keep]


def invcdf(c, t, u):
    """griddedInterpolant(c, t) evaluated at u: linear, linear extrapolation."""
    u = np.asarray(u, dtype=float)
    i = np.clip(np.searchsorted(c, u, side="right") - 1, 0, len(c) - 2)
    return t[i] + (u - c[i]) / (c[i + 1] - c[i]) * (t[i + 1] - t[i])


def prepare_sigma(d, acoustics, freq, v, cv, corr, acf, lc, nu=None, sigma=None, nth=1_000_000):
    """prepareSigma (MaterialClass.m:2379-2442); returns a dict of tables and scalars."""
    if sigma is None:
        sigma = sigma_functions(d, acoustics, freq, v, cv, corr, acf, lc, nu)
    out = {}
    if acoustics:
        S, Sp, c, t = prepare_sigma_one(sigma[0], d, nth)
        out.update(Sigma=S, Sigmapr=Sp, tables=[(c, t)])
        out["Diffusivity"] = v ** 2 / (d * (S - Sp))
        out["meanFreeTime"] = np.array([1 / S, 1 / S])
        out["meanFreePath"] = v / S
        out["transportMeanFreePath"] = d * out["Diffusivity"] / v
        out["g"] = 1 - out["meanFreePath"] / out["transportMeanFreePath"]
        out["P2P"] = 1.0
        out["S2S"] = 1.0
        return out
    vp, vs = v
    S = np.zeros((2, 2))
    Sp = np.zeros((2, 2))
    tabs = []
    for i in range(2):
        for j in range(2):
            S[i, j], Sp[i, j], c, t = prepare_sigma_one(sigma[i][j], d, nth)
            tabs.append((c, t))
    mft = 1.0 / S.sum(axis=1)
    K = vp / vs
    den = (S[0, 0] + S[0, 1] - Sp[0, 0]) * (S[1, 1] + S[1, 0] - Sp[1, 1]) - Sp[0, 1] * Sp[1, 0]
    tP = (vp * (S[1, 1] + S[1, 0] - Sp[1, 1]) + vs * Sp[0, 1]) / den
    tS = (vs * (S[0, 0] + S[0, 1] - Sp[0, 0]) + vp * Sp[1, 0]) / den
    Dp, Ds = vp * tP / d, vs * tS / d
    out.update(Sigma=S, Sigmapr=Sp, tables=tabs, meanFreeTime=mft,
               meanFreePath=np.array([vp, vs]) * mft,
               transportMeanFreePath=np.array([tP, tS]),
               Diffusivity=(Dp + 2 * K ** 3 * Ds) / (1 + 2 * K ** 3),
               P2P=S[0, 0] / S[0].sum(), S2S=S[1, 1] / S[1].sum())
    return out


def zoeppritz_fluid(theta_deg, vp1, vs1, rho1, vp2=343.0, vs2=0.0, rho2=1.0):
    """ZoeppritzFluid.m:47-222 -> dict of energy coefficients on the given angle grid."""
    th = np.asarray(theta_deg, dtype=float) * np.pi / 180
    keys = ["E_Rpp", "E_Rpsv", "E_Tpp", "E_Rsvsv", "E_Rsp", "E_Tsp", "E_Rsh"]
    out = {k: np.zeros_like(th) for k in keys}
    casin = lambda x: np.arcsin(np.complex128(x))
    for i, a in enumerate(th):
        # P incidence
        p = math.sin(a) / vp1
        phi1 = complex(a)
        psi1 = casin(vs1 * p)
        phi2 = casin(vp2 * p)
        psi2 = casin(vs2 * p)
        M = np.array([
            [np.cos(phi1), -np.sin(psi1), np.cos(phi2)],
            [-np.cos(2 * psi1), vs1 / vp1 * np.sin(2 * psi1), (rho2 * vp2 / (rho1 * vp1)) * np.cos(2 * psi2)],
            [np.sin(2 * phi1), vp1 / vs1 * np.cos(2 * psi1),
             (rho2 * vp1 * vs2 * vs2 / (rho1 * vp2 * vs1 * vs1)) * np.sin(2 * phi2)]], dtype=complex)
        psi0 = casin(vs1 * math.sin(a) / vp1)
        F = np.array([math.cos(a), np.cos(2 * psi0), math.sin(2 * a)], dtype=complex)
        R = np.linalg.solve(M, F)
        out["E_Rpp"][i] = abs(R[0]) ** 2
        out["E_Rpsv"][i] = (rho1 * vs1 * np.cos(psi1).real) / (rho1 * vp1 * np.cos(phi1).real) * abs(R[1]) ** 2
        out["E_Tpp"][i] = (rho2 * vp2 * np.cos(phi2).real) / (rho1 * vp1 * np.cos(phi1).real) * abs(R[2]) ** 2
        if a == 0:
            out["E_Rpsv"][i] = 0.0
        # SV incidence
        p = math.sin(a) / vs1
        phi1 = casin(vp1 * p)
        psi1 = complex(a)
        phi2 = casin(vp2 * p)
        psi2 = casin(vs2 * p)
        M = np.array([
            [np.cos(phi1), -np.sin(psi1), np.cos(phi2)],
            [-np.cos(2 * psi1), vs1 / vp1 * np.sin(2 * psi1), (rho2 * vp2 / (rho1 * vp1)) * np.cos(2 * psi2)],
            [np.sin(2 * phi1), (vp1 / vs1) * np.cos(2 * psi1),
             (rho2 * vp1 * vs2 * vs2 / (rho1 * vp2 * vs1 * vs1)) * np.sin(2 * phi2)]], dtype=complex)
        F = np.array([-math.sin(a), -vs1 * math.sin(2 * a) / vp1, vp1 * math.cos(2 * a) / vs1], dtype=complex)
        R = np.linalg.solve(M, F)
        out["E_Rsp"][i] = (rho1 * vp1 * np.cos(phi1).real) / (rho1 * vs1 * np.cos(psi1).real) * abs(R[0]) ** 2
        out["E_Rsvsv"][i] = abs(R[1]) ** 2
        out["E_Tsp"][i] = (rho2 * vp2 * np.cos(phi2).real) / (rho1 * vs1 * np.cos(psi1).real) * abs(R[2]) ** 2
        if a == 0:
            out["E_Rsp"][i] = 0.0
        out["E_Rsh"][i] = 1.0
    return out
