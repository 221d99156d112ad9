"""GB300-native radiative-transfer Monte Carlo engine.

Drop-in for the hot path of cottereau/RadiativeTransferMonteCarlo:
``obs = radiativeTransfer(geometry, source, material, observation)`` with the transport
(initializeParticle + propagateParticleSmallDt + observeTime) on sm_103a CUDA kernels
behind the C ABI of librtmc (include/rtmc.h).
"""
from .adjoint import radiativeTransferGradient
from .material import MaterialClass
from .observation import colon, initialize_observation
from .radiative_transfer import (TransportProblem, build_problem, get_context, normalise, radiativeTransfer,
                                 run_transport)
from .resumable import radiative_transfer_resumable

__all__ = ["MaterialClass", "radiativeTransfer", "radiativeTransferGradient", "build_problem", "run_transport", "normalise",
           "initialize_observation", "colon", "TransportProblem", "get_context", "radiative_transfer_resumable"]
