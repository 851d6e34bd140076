from .result import Result
from .simulation import Simulation
from .measure import Measure

from .beam import BeamResult, BeamPropagationResult
from .si import SIResult
from .pdt import PDTResult, TrackedPDTResult
from .structure_function import StructureFunctionResult
from .wind import WindResult, TimeCoherenceResult, TimeBWcorrSimulation
