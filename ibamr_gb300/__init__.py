"""GB300-native Lagrangian-Eulerian interaction (IBAMR LEInteractor spread /
interpolate) -- Python host binding of libibx.  See include/ibx.h."""

from . import ibx  # noqa: F401
