"""torchsim_gb300 — the extended-phase-graph hot path of torchsim on GB300.

Public API kept from the reference (FiRMLAB-Pisa/torchsim):

* ``mrf_sim``, ``fse_sim`` — functional simulators with ``diff=`` Jacobians;
* ``MRFSimulator``, ``FSESimulator`` — ``simulate`` / ``jacobian``;
* ``SequenceDesign``, ``Bounded``, ``crlb`` — sequence design through the
  adjoint kernel.

All compute runs in hand-written sm_103a CUDA kernels behind the C ABI in
``include/torchsim_gb300.h``; there is no CPU fallback.
"""

from .design import Bounded, SequenceDesign, SequenceOptimization, crlb
from .simulators import FSESimulator, MRFSimulator, fse_sim, mrf_sim

__all__ = ["Bounded", "FSESimulator", "MRFSimulator", "SequenceDesign", "SequenceOptimization",
           "crlb", "fse_sim", "mrf_sim"]
__version__ = "0.1.0"
