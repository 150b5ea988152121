"""scone_gb300 -- GB300-native (sm_103a) Monte Carlo particle-tracking cycle with SCONE's
transportOperator / nuclearDatabase / tallyClerk contract behind a C ABI (include/scone_gpu.h)."""
from . import abi, problems  # noqa: F401
