"""clmgb — GB300-native soil/snow column solve (CLM5 SoilTemperature + moisture-form
Richards) behind a C ABI (include/clmgb.h); Python host mirror of CLM.jl's entry points."""
from . import abi  # noqa: F401
from .state import ColumnState  # noqa: F401

__all__ = ["abi", "ColumnState"]
