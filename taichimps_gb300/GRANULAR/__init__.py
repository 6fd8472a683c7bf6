from .base import GranularPair
from .granular import PairGranular, mix_stiffness_e, mix_stiffness_g
from .hertz import GranHertz
from .hertz_history import GranHertzHistory
from .hooke import GranHooke
from .hooke_history import GranHookeHistory

__all__ = ["GranularPair", "GranHooke", "GranHookeHistory", "GranHertz", "GranHertzHistory",
           "PairGranular", "mix_stiffness_e", "mix_stiffness_g"]
