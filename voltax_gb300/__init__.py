"""voltax_gb300: the voltax Newton inner loop on GB300 (sm_103a).

Device evaluation with deterministic stamping, supernodal sparse LU
refactorization under a reused symbolic plan, and level-scheduled
(transposed) triangular solves, all in hand-written CUDA behind a C ABI
(include/vxg.h), with drop-ins for ``voltax.dc``, ``voltax.transient`` and
``voltax.sparse``.
"""

from . import library, signals, sparse, workloads  # noqa: F401
from .analysis import (ACSolution, Options, Solution, ac, dc, dc_sweep,  # noqa: F401
                       linearize, time_grid, transient)
from .builder import CircuitBuilder  # noqa: F401
from .circuit import Circuit, Layout  # noqa: F401
from .elements import (VT_300K, Capacitor, Conductance, CurrentSource,  # noqa: F401
                       BJT, CCCS, CCVS, VCCS, VCVS, CoupledInductors, Diode, IdealOpAmp,
                       OpAmp, Switch,
                       Transformer, EKVMOSFET, Element, Inductor, Level1MOSFET,
                       MOSProcess, Resistor, VoltageSource, concatenate)

__version__ = "0.1.0"
