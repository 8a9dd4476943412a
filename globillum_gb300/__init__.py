"""GB300-native implementation of globillum's path-tracing hot path."""
