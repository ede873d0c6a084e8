"""torchsim_gb300 — the extended-phase-graph hot path of torchsim on GB300.

Public API kept from the reference (FiRMLAB-Pisa/torchsim):

* ``mrf_sim``, ``fse_sim`` — functional simulators with ``diff=`` Jacobians;
* ``MRFSimulator``, ``FSESimulator`` — ``simulate`` / ``jacobian``;
* ``EpgEngine().simulate(events, tissue)`` — a packed stream on the kernels,
  with its sample labels (``SimulationResult``);
* ``SequenceDesign``, ``Bounded``, ``crlb`` — sequence design through the
  adjoint kernel;
* ``DictionaryMatcher``, ``MatchResult`` — dictionary matching on the tensor
  cores;
* ``NonlinearLeastSquares``, ``GaussNewton``, ``TrustRegion``,
  ``ModelOperator`` — voxel-wise mapping (Levenberg-Marquardt) on the fused
  normal-equation sweep.

All compute runs in hand-written sm_103a CUDA kernels behind the C ABI in
``include/torchsim_gb300.h``; there is no CPU fallback.
"""

from .design import Bounded, SequenceDesign, SequenceOptimization, crlb
from . import recon, serving
from .matching import DictionaryMatcher, MatchResult
from .recon import GaussNewton, ModelOperator, NonlinearLeastSquares, TrustRegion
from .simulators import (EpgEngine, FSESimulator, MRFSimulator, SimulationResult, fse_sim,
                         mrf_sim)

__all__ = ["Bounded", "DictionaryMatcher", "EpgEngine", "FSESimulator", "GaussNewton",
           "MRFSimulator", "MatchResult", "ModelOperator", "NonlinearLeastSquares",
           "SequenceDesign", "SequenceOptimization", "SimulationResult", "TrustRegion", "crlb",
           "fse_sim", "mrf_sim"]
__version__ = "0.1.0"
