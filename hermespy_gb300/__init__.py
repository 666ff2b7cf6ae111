"""GB300 Monte Carlo link engine for HermesPy's OFDM fading-link drop loop.

The package mirrors the reference's plugin classes on the hot path
(``MultipathFadingChannel`` realize/sample/propagate/state, ``OFDMWaveform``
map/place/modulate/demodulate/pick/unmap, the channel estimation and
equalization classes, AWGN and noise levels, ``BitErrorEvaluator``) on top of
hand-written sm_103a CUDA kernels reached through the C ABI of ``libhpx.so``
(``include/hpx.h``), and adds the batched ``LinkEngine``. There is no CPU
fallback: the classes raise if the library or a CUDA device is missing.
"""

from .channel import (
    ChannelStateInformation,
    CustomAntennaCorrelation,
    Exponential,
    ExponentialAntennaCorrelation,
    LinkState,
    MultipathFadingChannel,
    MultipathFadingRealization,
    MultipathFadingSample,
)
from .containers import DenseSignal, Signal, SignalBlock, SparseSignal, StatedSymbols, Symbols
from .engine import BerPoint, LinkEngine, clopper_pearson
from .estimation import (
    ChannelEqualization,
    ChannelEstimation,
    LinearMinimumMeanSquareErrorChannelEqualization,
    OFDMIdealChannelEstimation,
    OrthogonalLeastSquaresChannelEstimation,
    OrthogonalLinearMinimumMeanSquareErrorChannelEqualization,
    OrthogonalZeroForcingChannelEqualization,
    ZeroForcingChannelEqualization,
    ls_interpolation_table,
)
from .fec import Encoder, EncoderManager, LDPCCoding
from .mapping import PskQamMapping
from .noise import AWGN, EBN0, ESN0, SNR, AWGNRealization
from .presets import TDL, CorrelationType, Cost259, Cost259Type, DeviceType, StandardAntennaCorrelation, TDLType
from .simulation import (
    BitErrorEvaluator,
    RandomBitsSource,
    SimplexLink,
    SimulatedDevice,
    SimulationScenario,
)
from .synchronization import (
    CorrelationSynchronization,
    OFDMCorrelationSynchronization,
    OFDMSynchronization,
    SchmidlCoxSynchronization,
    Synchronization,
)
from .waveform import (
    ElementType,
    GridElement,
    GridResource,
    OFDMWaveform,
    PilotSection,
    PrefixType,
    SchmidlCoxPilotSection,
    SymbolSection,
)

__version__ = "1.0.0"
