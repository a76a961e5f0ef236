"""GB300-native exact negacyclic multiplier (drop-in for ByteCRT's fherma_* path)."""
from . import inputs  # noqa: F401
