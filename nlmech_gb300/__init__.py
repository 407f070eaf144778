"""GB300-native peridynamics hot path (NLMech drop-in)."""
