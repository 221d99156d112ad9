"""MaterialClass: material description and FP64 scattering tables.

Mirrors @MaterialClass/MaterialClass.m of cottereau/RadiativeTransferMonteCarlo for what
the transport needs: the constructor (:59-97), the SpectralLaw validation (:138-140),
preset (:1765-1785), prepareSigma (:2379-2442) and Zoeppritz (:1786-1885).  The tables
are built by the C++ FP64 builder of librtmc (rtmc_tables_build).
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib

SPECTRAL_LAWS = ("", "exp", "power_law", "gaussian", "triangular", "low_pass", "VonKarman",
                 "monodispersesphere", "image", "Imported")
_BUILDABLE = ("exp", "power_law", "gaussian", "triangular", "low_pass", "VonKarman")


def validatestring(value: str, options) -> str:
    """Case-insensitive prefix match, as MATLAB's validatestring (MaterialClass.m:138-140)."""
    v = value.lower()
    exact = [o for o in options if o.lower() == v]
    if exact:
        return exact[0]
    hits = [o for o in options if o.lower().startswith(v)]
    if len(hits) == 1:
        return hits[0]
    if hits:
        shortest = min(hits, key=len)
        if all(h.lower().startswith(shortest.lower()) for h in hits):
            return shortest
    raise ValueError(f"Expected input to match one of these values: {', '.join(o for o in options if o)}; "
                     f"the input, '{value}', did not match uniquely.")


class MaterialClass:
    """Material properties and differential scattering cross-sections."""

    def __init__(self, geometry=None, freq=None, acoustics=None, v=None, coefficients_of_variation=None,
                 correlation_coefficients=None, acf=None, lc=None):
        self.d = 3
        self.type = "isotropic"
        self.acoustics = None
        self.v = None
        self.vp = None
        self.vs = None
        self.rho = None
        self.Frequency = None
        self.Q = math.inf
        self.coefficients_of_variation = None
        self.correlation_coefficients = None
        self._spectral_law = ""
        self.SpectralParam = {}
        self.CorrelationLength = None
        self.sigma = None  # constant cross-sections (numbers): [s] acoustic, [[PP, PS], [SP, SS]] elastic
        self.Sigma = None
        self.Sigmapr = None
        self.invcdf = None  # librtmc tables handle
        self.Diffusivity = None
        self.meanFreeTime = None
        self.meanFreePath = None
        self.transportMeanFreeTime = None
        self.transportMeanFreePath = None
        self.g = None
        self.P2P = None
        self.S2S = None
        self.timeSteps = 0
        if geometry is not None:
            d = geometry["dimension"]
            if d == 1:
                raise ValueError("Total scattering cross-sections for 1D case are to be implemented in future releases")
            self.d = int(d)
            self.acoustics = bool(acoustics)
            self.Frequency = freq
            if self.acoustics:
                self.v = float(np.atleast_1d(v)[0])
            else:
                self.vp, self.vs = float(v[0]), float(v[1])
            self.coefficients_of_variation = np.atleast_1d(np.asarray(coefficients_of_variation, dtype=float))
            self.correlation_coefficients = np.atleast_1d(np.asarray(correlation_coefficients, dtype=float))
            self.CorrelationLength = lc
            self.SpectralLaw = acf

    @property
    def SpectralLaw(self):
        return self._spectral_law

    @SpectralLaw.setter
    def SpectralLaw(self, value):
        self._spectral_law = validatestring(value, SPECTRAL_LAWS)

    # -- MaterialClass.preset (MaterialClass.m:1765-1785)
    @staticmethod
    def preset(n: int) -> "MaterialClass":
        m = MaterialClass()
        if n == 1:
            m.sigma = [1 / 4 / math.pi]
            m.v = 2.0
            m.acoustics = True
        elif n == 2:
            m.sigma = [1 / 10 / math.pi]
            m.v = 2.0
            m.acoustics = True
        elif n in (3, 4):
            m.vp = 6.0
            m.vs = 6 / math.sqrt(3)
            m.acoustics = False
        else:
            raise ValueError("unknown preset")
        return m

    def _descriptor(self, d: int) -> _lib.RtmcMaterial:
        md = _lib.RtmcMaterial()
        md.d = int(d)
        md.acoustics = 1 if self.acoustics else 0
        md.n_theta = 1_000_000
        if self.acoustics:
            md.v[0] = float(self.v) if self.v is not None else 0.0
        else:
            md.v[0], md.v[1] = float(self.vp), float(self.vs)
        if self.sigma is not None:
            flat = np.asarray(self.sigma, dtype=float).ravel()
            want = 1 if self.acoustics else 4
            if flat.size != want:
                raise ValueError("constant sigma needs 1 (acoustic) or 2x2 (elastic) values")
            md.psdf = _lib.PSDF["const"]
            for i, s in enumerate(flat):
                md.sigma_const[i] = s
            return md
        law = self.SpectralLaw
        if law not in _BUILDABLE:
            raise NotImplementedError(f"SpectralLaw '{law}' has no table builder here")
        md.psdf = _lib.PSDF[law]
        if not (self.Frequency and self.CorrelationLength):
            raise ValueError("Frequency and CorrelationLength are required to compute cross-sections")
        md.freq = float(np.atleast_1d(self.Frequency)[0])
        md.lc = float(self.CorrelationLength)
        cv = np.atleast_1d(self.coefficients_of_variation).astype(float)
        corr = np.atleast_1d(self.correlation_coefficients).astype(float)
        need = 2 if self.acoustics else 3
        if cv.size < need:
            raise ValueError(f"coefficients_of_variation needs {need} values")
        if corr.size < (1 if self.acoustics else 3):
            raise ValueError("correlation_coefficients needs 1 (acoustic) or 3 (elastic) values")
        for i in range(need):
            md.cv[i] = cv[i]
        for i in range(1 if self.acoustics else 3):
            md.corr[i] = corr[i]
        if not self.acoustics:
            rlm, rlr, rmr = corr[:3]
            Cc = np.array([[1, rlm, rlr], [rlm, 1, rmr], [rlr, rmr, 1]])
            if np.linalg.eigvalsh(Cc).min() < -1e-12:
                raise ValueError("The lambda-mu-rho correlation matrix is not positive semidefinite.")
        if law == "VonKarman":
            if "nu" not in self.SpectralParam:
                raise ValueError("Please add the Hurst number for VonKarman PSDF")
            md.nu = float(self.SpectralParam["nu"])
        return md

    # -- MaterialClass.prepareSigma (MaterialClass.m:2379-2442)
    @staticmethod
    def prepareSigma(mat: "MaterialClass", d: int) -> "MaterialClass":
        tables = _lib.Tables.build(mat._descriptor(d))
        info = tables.info()
        mat.invcdf = tables
        if mat.acoustics:
            mat.Sigma = info.Sigma[0]
            mat.Sigmapr = info.Sigmapr[0]
            mat.Diffusivity = info.diffusivity
            mat.meanFreeTime = info.mean_free_time[0]
            mat.meanFreePath = mat.v * mat.meanFreeTime
            mat.transportMeanFreePath = info.transport_mean_free_path[0]
            mat.transportMeanFreeTime = mat.transportMeanFreePath / mat.v
            mat.g = info.g
            mat.vp = mat.v
            mat.vs = 0.0
            mat.P2P = mat.S2S = 1.0
        else:
            mat.Sigma = np.array(info.Sigma[:]).reshape(2, 2)
            mat.Sigmapr = np.array(info.Sigmapr[:]).reshape(2, 2)
            mat.meanFreeTime = np.array(info.mean_free_time[:])
            mat.meanFreePath = np.array([mat.vp, mat.vs]) * mat.meanFreeTime
            mat.transportMeanFreePath = np.array(info.transport_mean_free_path[:])
            mat.transportMeanFreeTime = mat.transportMeanFreePath / np.array([mat.vp, mat.vs])
            mat.Diffusivity = info.diffusivity
            mat.P2P = info.p2p
            mat.S2S = info.s2s
        return mat

    # -- MaterialClass.Zoeppritz (MaterialClass.m:1786-1885): solid / air, air in SI units
    @staticmethod
    def Zoeppritz(mat: "MaterialClass") -> dict:
        if mat.acoustics:
            raise ValueError("This dont work for acoustic material")
        if mat.rho is None:
            raise ValueError("Please define the density in MaterialClass before calling MaterialInterface.")
        j1 = np.linspace(0.0, 90.0, 181)
        out = _lib.zoeppritz_fluid(j1, mat.vp, mat.vs, float(mat.rho), 343.0, 0.0, 1.0)
        out["j1_deg"] = j1
        return out
