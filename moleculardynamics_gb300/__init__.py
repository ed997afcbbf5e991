"""GB300-native MD step engine for vakuras/moleculardynamics (see include/mdgb.h)."""
